// Off-fault plasticity: Drucker-Prager yield check at the nodes of a nodal basis and the
// viscoplastic return map of the stresses (Plasticity.cpp:47-214, Wollherr et al. 2018, eqs. 10-13),
// with the plastic strain and its accumulated norm eta.  One kernel per order, FP32.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "output.h"

namespace sei {
namespace {

constexpr int kPlCells = 32;  // cells per CTA; thread (stress component q < 6, cell lane)

// A CTA of 192 threads: V and Vinv staged in shared memory (rows padded to Bp floats, read as
// broadcast float4); the nodal stresses of 32 cells S [6][B][32] exchanged between the column
// threads (q, lane) and the node threads (nodes q, q + 6, ... of cell lane).
template <int B>
__global__ void __launch_bounds__(6 * kPlCells) sei_plasticity(PlasticityArgs a) {
  constexpr int Bp = (B + 3) / 4 * 4;
  extern __shared__ float4 sm4[];
  float* V = reinterpret_cast<float*>(sm4);  // [B][Bp]
  float* Vi = V + B * Bp;                     // [B][Bp]
  float* S = Vi + B * Bp;                     // [6][B][32]
  __shared__ int adjust[kPlCells];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    const float4* src = reinterpret_cast<const float4*>(a.mats);
    for (int i = threadIdx.x; i < 2 * B * Bp / 4; i += blockDim.x) sm4[i] = src[i];
  }
  if (threadIdx.x < kPlCells) adjust[threadIdx.x] = 0;
  const int64_t cell = a.begin + (int64_t)blockIdx.x * kPlCells + lane;
  const bool valid = cell < a.end;
  const int64_t cl = valid ? cell : a.end - 1;
  float col[Bp];
  sei_load_col<Bp>(a.Q + ((size_t)cl * 9 + q) * Bp, col);
  __syncthreads();

  // nodal stresses plus the initial loading: S[q][n] = sum_k V[n][k] Q[q][k] + s0[q][n]
  // per-node arrays are tiled [cell / 32][K][B][32]: a warp's cells read one node as one run
  const size_t tile = (size_t)(cl >> 5), tl = (size_t)(cl & 31);
  const float* s0 = a.s0 + (tile * 6 + q) * B * 32 + tl;
  float* Sq = S + q * B * kPlCells + lane;
#pragma unroll
  for (int n0 = 0; n0 < B; n0 += 4) {
    float acc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = (n0 + j < B) ? __ldg(s0 + (n0 + j) * 32) : 0.f;
#pragma unroll
    for (int k = 0; k < Bp; k += 4) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (n0 + j < B) {
          const float4 v = *reinterpret_cast<const float4*>(V + (n0 + j) * Bp + k);
          acc[j] = fmaf(v.x, col[k], acc[j]);
          acc[j] = fmaf(v.y, col[k + 1], acc[j]);
          acc[j] = fmaf(v.z, col[k + 2], acc[j]);
          acc[j] = fmaf(v.w, col[k + 3], acc[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (n0 + j < B) Sq[(n0 + j) * kPlCells] = acc[j];
  }
  __syncthreads();

  // at each node: mean stress, deviator, tau = sqrt(J2), tau_c; the yield factor and, where
  // tau > tau_c, the stress update (the deviator times the factor) and the plastic strain rate
  int any = 0;
  const float fac = valid ? __ldg(a.mufac + cl) * a.inv_tvr : 0.f;
  for (int n = q; n < B; n += 6) {
    float s[6];
#pragma unroll
    for (int x = 0; x < 6; ++x) s[x] = S[(x * B + n) * kPlCells + lane];
    const float m = (s[0] + s[1] + s[2]) * (1.f / 3.f);
    s[0] -= m;
    s[1] -= m;
    s[2] -= m;
    const float j2 = 0.5f * (s[0] * s[0] + s[1] * s[1] + s[2] * s[2]) + s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    const float tau = sqrtf(j2);
    const size_t at = (tile * B + n) * 32 + tl;
    const float lim = fmaxf(0.f, __ldg(a.ccos + at) - m * __ldg(a.ssin + at));
    if (valid && tau > lim) {
      any = 1;
      const float y = (lim / tau - 1.f) * a.relax;
      float* ps = a.pstrain + (tile * 7 * B + n) * 32 + tl;
      float sq = 0.f;
#pragma unroll
      for (int x = 0; x < 6; ++x) {
        const float u = s[x] * y;
        const float rate = -fac * u;
        ps[x * B * 32] += a.dt * rate;
        sq = fmaf(rate, rate, sq);
        S[(x * B + n) * kPlCells + lane] = u;
      }
      ps[6 * B * 32] += a.dt * sqrtf(0.5f * sq);
    } else {
#pragma unroll
      for (int x = 0; x < 6; ++x) S[(x * B + n) * kPlCells + lane] = 0.f;
    }
  }
  if (any) adjust[lane] = 1;
  __syncthreads();

  // modal update of the yielding cells: Q[q][k] += sum_n Vinv[k][n] S[q][n]
  if (!valid || !adjust[lane]) return;
  float u[Bp];
#pragma unroll
  for (int n = 0; n < Bp; ++n) u[n] = n < B ? Sq[n * kPlCells] : 0.f;
#pragma unroll
  for (int k = 0; k < B; ++k) {
    float acc = col[k];
#pragma unroll
    for (int n = 0; n < Bp; n += 4) {
      const float4 v = *reinterpret_cast<const float4*>(Vi + k * Bp + n);
      acc = fmaf(v.x, u[n], acc);
      acc = fmaf(v.y, u[n + 1], acc);
      acc = fmaf(v.z, u[n + 2], acc);
      acc = fmaf(v.w, u[n + 3], acc);
    }
    col[k] = acc;
  }
  sei_store_col<Bp>(a.Q + ((size_t)cell * 9 + q) * Bp, col);
  if (q == 0) atomicAdd(a.yield, 1ull);
}

template <int B>
int launchB(const PlasticityArgs& a, cudaStream_t s) {
  constexpr int Bp = (B + 3) / 4 * 4;
  const size_t smem = sizeof(float) * (2 * B * Bp + 6 * B * kPlCells);
  if (cudaFuncSetAttribute(sei_plasticity<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  const int64_t n = a.end - a.begin;
  const int64_t blocks = (n + kPlCells - 1) / kPlCells;
  if (blocks > 0x7fffffff) return -1;
  sei_plasticity<B><<<(unsigned)blocks, 6 * kPlCells, smem, s>>>(a);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

int launchPlasticity(int order, const PlasticityArgs& a, void* stream) {
  if (a.end <= a.begin) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (order) {
    case 4:
      return launchB<20>(a, s);
    case 5:
      return launchB<35>(a, s);
    case 6:
      return launchB<56>(a, s);
    default:
      return -1;
  }
}

bool plasticityMatrices(int order, const double* nodes, std::vector<double>& v, std::vector<double>& vinv) {
  const int B = numBasis(order);
  const double identity[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  std::vector<double> phi(B), dphi((size_t)3 * B);
  v.assign((size_t)B * B, 0.0);
  for (int n = 0; n < B; ++n) {
    basisAtPoint(order, nodes + 3 * n, identity, phi.data(), dphi.data());
    for (int k = 0; k < B; ++k) v[(size_t)n * B + k] = phi[k];
  }
  // Gauss-Jordan elimination with partial pivoting on [V | I]
  std::vector<double> a(v);
  vinv.assign((size_t)B * B, 0.0);
  for (int i = 0; i < B; ++i) vinv[(size_t)i * B + i] = 1.0;
  double scale = 0.0;
  for (double x : a) scale = std::fmax(scale, std::fabs(x));
  for (int c = 0; c < B; ++c) {
    int p = c;
    for (int r = c + 1; r < B; ++r)
      if (std::fabs(a[(size_t)r * B + c]) > std::fabs(a[(size_t)p * B + c])) p = r;
    const double piv = a[(size_t)p * B + c];
    if (!(std::fabs(piv) > 1e-12 * scale)) return false;
    if (p != c)
      for (int k = 0; k < B; ++k) {
        std::swap(a[(size_t)p * B + k], a[(size_t)c * B + k]);
        std::swap(vinv[(size_t)p * B + k], vinv[(size_t)c * B + k]);
      }
    for (int k = 0; k < B; ++k) {
      a[(size_t)c * B + k] /= piv;
      vinv[(size_t)c * B + k] /= piv;
    }
    for (int r = 0; r < B; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * B + c];
      if (f == 0.0) continue;
      for (int k = 0; k < B; ++k) {
        a[(size_t)r * B + k] -= f * a[(size_t)c * B + k];
        vinv[(size_t)r * B + k] -= f * vinv[(size_t)c * B + k];
      }
    }
  }
  return true;
}

void latticeNodes(int order, double* nodes) {
  const int d = order - 1;
  int n = 0;
  for (int k = 0; k <= d; ++k)
    for (int j = 0; j + k <= d; ++j)
      for (int i = 0; i + j + k <= d; ++i) {
        nodes[3 * n] = d ? (double)i / d : 0.25;
        nodes[3 * n + 1] = d ? (double)j / d : 0.25;
        nodes[3 * n + 2] = d ? (double)k / d : 0.25;
        ++n;
      }
}

}  // namespace sei
