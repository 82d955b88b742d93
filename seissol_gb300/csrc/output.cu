// Output path: receivers (src/Kernels/Receiver.cpp:118-214, src/ResultWriter/ReceiverWriter.cpp)
// and the device -> host staging shared with the fault output.
//
// A receiver is evaluated at the start of each step of its cell: the CK derivatives of the
// receiver cells (the ADER kernel on a compact copy of those cells) give the Taylor expansion
// in time, evaluated at every sampling time inside the step, then projected onto the basis
// functions at the receiver point (and their gradients for rotation and strain).  Rows go into a
// device ring of two halves; a full half is copied on the stager's stream into pinned memory,
// and a host function appends it to the host store, so the copies overlap the following steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "output.h"

namespace {

__global__ void sei_gather_rows(int m, const int32_t* __restrict__ src, const float* __restrict__ in,
                                float* __restrict__ out, int rowFloats) {
  const int64_t total = (int64_t)m * rowFloats;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / rowFloats, k = e % rowFloats;
    out[e] = __ldg(in + (int64_t)src[r] * rowFloats + k);
  }
}

// One warp per receiver.  Row of sample s: time, the quantities of qmask, then rotation
// (d8/dy - d7/dz, d6/dz - d8/dx, d7/dx - d6/dy) and strain (eps_xx, eps_xy, eps_xz, eps_yy,
// eps_yz, eps_zz from the velocity gradient), Receiver.cpp:271-302.
template <int N, bool VIS>
__global__ void __launch_bounds__(128) sei_recv_eval(sei::RecvEvalArgs A) {
  constexpr int B = N * (N + 1) * (N + 2) / 6;
  constexpr int L = (B + 31) / 32;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= A.nrecv) return;
  const int r = A.list[warp];
  int dsz = VIS ? N * 27 * B : 0;
#pragma unroll
  for (int i = 0; i < N; ++i) dsz += VIS ? 0 : (N - i) * (N - i + 1) * (N - i + 2) / 6 * 9;
  const float* d = A.derivs + (size_t)A.slot[r] * dsz;
  float phi[L], dphi[L][3];
#pragma unroll
  for (int u = 0; u < L; ++u) {
    const int l = lane + 32 * u;
    const bool on = l < B;
    phi[u] = on ? A.phi[(size_t)r * B + l] : 0.f;
#pragma unroll
    for (int x = 0; x < 3; ++x) dphi[u][x] = on && A.derived ? A.dphi[((size_t)r * 3 + x) * B + l] : 0.f;
  }
  for (int s = 0; s < A.nsamples; ++s) {
    // Taylor coefficients t^i / i! at the sample's offset from the expansion point
    float co[N];
    const float t = (float)A.offset[s];
    co[0] = 1.f;
#pragma unroll
    for (int i = 1; i < N; ++i) co[i] = co[i - 1] * t / (float)i;
    float val[9], grad[3][3];
#pragma unroll
    for (int q = 0; q < 9; ++q) val[q] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int x = 0; x < 3; ++x) grad[a][x] = 0.f;
#pragma unroll
    for (int u = 0; u < L; ++u) {
      const int l = lane + 32 * u;
      if (l >= B) continue;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        float v = 0.f;
        int off = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          // the elastic kernels keep the rows of degree < N - i of stage i; the viscoelastic ones all
          const int bi = VIS ? B : (N - i) * (N - i + 1) * (N - i + 2) / 6;
          if (l < bi) v = fmaf(co[i], __ldg(d + off + q * bi + l), v);
          off += (VIS ? 27 : 9) * bi;
        }
        val[q] = fmaf(phi[u], v, val[q]);
        if (q >= 6)
#pragma unroll
          for (int x = 0; x < 3; ++x) grad[q - 6][x] = fmaf(dphi[u][x], v, grad[q - 6][x]);
      }
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
#pragma unroll
      for (int q = 0; q < 9; ++q) val[q] += __shfl_xor_sync(0xffffffffu, val[q], m);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int x = 0; x < 3; ++x) grad[a][x] += __shfl_xor_sync(0xffffffffu, grad[a][x], m);
    }
    if (lane == 0) {
      double* row = A.out + ((size_t)s * A.nrecv + warp) * A.ncols;
      int c = 0;
      row[c++] = A.time0 + A.offset[s];
      for (int q = 0; q < 9; ++q)
        if (A.qmask & (1u << q)) row[c++] = val[q];
      if (A.derived & SEI_RECV_ROTATION) {
        row[c++] = grad[2][1] - grad[1][2];
        row[c++] = grad[0][2] - grad[2][0];
        row[c++] = grad[1][0] - grad[0][1];
      }
      if (A.derived & SEI_RECV_STRAIN) {
        row[c++] = grad[0][0];
        row[c++] = 0.5f * (grad[0][1] + grad[1][0]);
        row[c++] = 0.5f * (grad[0][2] + grad[2][0]);
        row[c++] = grad[1][1];
        row[c++] = 0.5f * (grad[1][2] + grad[2][1]);
        row[c++] = grad[2][2];
      }
    }
  }
}

// ---- Dubiner basis on the host with exact gradients (value and three partials) ----
struct Dual {
  double v, d[3];
};
Dual dconst(double c) { return {c, {0, 0, 0}}; }
Dual operator+(const Dual& a, const Dual& b) { return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; }
Dual operator-(const Dual& a, const Dual& b) { return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; }
Dual operator*(const Dual& a, const Dual& b) {
  return {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}
Dual operator*(double s, const Dual& a) { return {s * a.v, {s * a.d[0], s * a.d[1], s * a.d[2]}}; }

// y^n P_n^(a,b)(x / y) by the three-term recurrence of the Jacobi polynomials, homogenised so that
// no division by y occurs (the collapsed coordinates of the tetrahedron).
Dual scaledJacobi(int n, double a, double b, const Dual& x, const Dual& y) {
  if (n == 0) return dconst(1.0);
  Dual pm1 = dconst(1.0);
  Dual pm = (0.5 * a - 0.5 * b) * y + (1.0 + 0.5 * (a + b)) * x;
  for (int m = 2; m <= n; ++m) {
    const Dual pm2 = pm1;
    pm1 = pm;
    const double c0 = 2.0 * m + a + b;
    const Dual t = (a * a - b * b) * y + (c0 * (c0 - 2.0)) * x;
    pm = (1.0 / (2.0 * m * (m + a + b) * (c0 - 2.0))) *
         ((c0 - 1.0) * (t * pm1) - (2.0 * (m + a - 1.0) * (m + b - 1.0) * c0) * (y * y * pm2));
  }
  return pm;
}

}  // namespace

namespace sei {

// ---- staging ----
Stager::~Stager() { release(); }

void Stager::release() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (int h = 0; h < 2; ++h) {
    if (dev_[h]) cudaFree(dev_[h]);
    if (host_[h]) cudaFreeHost(host_[h]);
    if (done_[h]) cudaEventDestroy(done_[h]);
    if (full_[h]) cudaEventDestroy(full_[h]);
    dev_[h] = host_[h] = nullptr;
    done_[h] = full_[h] = nullptr;
  }
  if (stream_) cudaStreamDestroy(stream_);
  stream_ = nullptr;
  rowBytes_ = rowsPerHalf_ = used_ = 0;
  std::lock_guard<std::mutex> g(mu_);
  store_.clear();
}

int Stager::init(size_t rowBytes, size_t rowsPerHalf) {
  release();
  rowBytes_ = rowBytes;
  rowsPerHalf_ = rowsPerHalf;
  const size_t bytes = rowBytes * rowsPerHalf;
  if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) return -1;
  for (int h = 0; h < 2; ++h) {
    if (cudaMalloc(&dev_[h], bytes) != cudaSuccess || cudaMallocHost(&host_[h], bytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&done_[h], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&full_[h], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      release();
      return -1;
    }
    cudaEventRecord(done_[h], stream_);
  }
  half_ = 0;
  used_ = 0;
  return 0;
}

struct StagerAppend {
  Stager* s;
  int half;
  size_t bytes;
};

void CUDART_CB Stager::appendHost(void* p) {
  StagerAppend* a = static_cast<StagerAppend*>(p);
  {
    std::lock_guard<std::mutex> g(a->s->mu_);
    const char* src = static_cast<const char*>(a->s->host_[a->half]);
    a->s->store_.insert(a->s->store_.end(), src, src + a->bytes);
  }
  delete a;
}

int Stager::flush(cudaStream_t compute) {
  if (used_ == 0) return 0;
  const size_t bytes = used_ * rowBytes_;
  const int h = half_;
  // the copy waits for the rows' producers; the next writes into this half wait for the copy
  if (cudaEventRecord(full_[h], compute) != cudaSuccess || cudaStreamWaitEvent(stream_, full_[h], 0) != cudaSuccess ||
      cudaMemcpyAsync(host_[h], dev_[h], bytes, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return -1;
  StagerAppend* a = new StagerAppend{this, h, bytes};
  if (cudaLaunchHostFunc(stream_, appendHost, a) != cudaSuccess) {
    delete a;
    return -1;
  }
  if (cudaEventRecord(done_[h], stream_) != cudaSuccess) return -1;
  half_ ^= 1;
  used_ = 0;
  // writes into the other half wait until its last copy finished
  return cudaStreamWaitEvent(compute, done_[half_], 0) == cudaSuccess ? 0 : -1;
}

void* Stager::reserve(size_t rows, cudaStream_t compute, int* err) {
  *err = 0;
  if (rows > rowsPerHalf_) {
    *err = -2;
    return nullptr;
  }
  if (used_ + rows > rowsPerHalf_ && flush(compute) != 0) {
    *err = -1;
    return nullptr;
  }
  void* p = static_cast<char*>(dev_[half_]) + used_ * rowBytes_;
  used_ += rows;
  return p;
}

int Stager::drain(cudaStream_t compute, void* out, size_t maxRows, size_t* nrows) {
  if (flush(compute) != 0) return -1;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -1;
  std::lock_guard<std::mutex> g(mu_);
  const size_t have = store_.size() / (rowBytes_ ? rowBytes_ : 1);
  const size_t take = std::min(have, maxRows);
  if (out && take) std::memcpy(out, store_.data(), take * rowBytes_);
  store_.erase(store_.begin(), store_.begin() + (ptrdiff_t)(take * rowBytes_));
  *nrows = take;
  return 0;
}

size_t Stager::pendingRows(cudaStream_t compute) {
  if (flush(compute) != 0) return 0;
  cudaStreamSynchronize(stream_);
  std::lock_guard<std::mutex> g(mu_);
  return rowBytes_ ? store_.size() / rowBytes_ : 0;
}

// ---- receivers ----
int launchGatherRows(int m, const int32_t* src, const float* in, float* out, int rowFloats, void* stream) {
  if (m <= 0) return 0;
  const int64_t total = (int64_t)m * rowFloats;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  sei_gather_rows<<<blocks, 256, 0, (cudaStream_t)stream>>>(m, src, in, out, rowFloats);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchRecvEval(int order, const RecvEvalArgs& a, void* stream) {
  if (a.nrecv <= 0 || a.nsamples <= 0) return 0;
  const int blocks = (a.nrecv + 3) / 4;
  cudaStream_t st = (cudaStream_t)stream;
  switch (order * 2 + (a.visco ? 1 : 0)) {
    case 4: sei_recv_eval<2, false><<<blocks, 128, 0, st>>>(a); break;
    case 6: sei_recv_eval<3, false><<<blocks, 128, 0, st>>>(a); break;
    case 8: sei_recv_eval<4, false><<<blocks, 128, 0, st>>>(a); break;
    case 9: sei_recv_eval<4, true><<<blocks, 128, 0, st>>>(a); break;
    case 10: sei_recv_eval<5, false><<<blocks, 128, 0, st>>>(a); break;
    case 11: sei_recv_eval<5, true><<<blocks, 128, 0, st>>>(a); break;
    case 12: sei_recv_eval<6, false><<<blocks, 128, 0, st>>>(a); break;
    default: return -1;
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

void basisAtPoint(int order, const double xez[3], const double grad[3][3], double* phi, double* dphi) {
  // grad[r] = d(xi_r)/dx (rows of the inverse Jacobian); dphi [3][B] in global coordinates
  const int B = numBasis(order);
  Dual xi{xez[0], {1, 0, 0}}, eta{xez[1], {0, 1, 0}}, zeta{xez[2], {0, 0, 1}};
  const Dual one = dconst(1.0);
  int l = 0;
  for (int o = 0; o < order; ++o)
    for (int k = 0; k <= o; ++k)
      for (int j = 0; j <= o - k; ++j) {
        const int i = o - j - k;  // reference ordering (Numerical/BasisFunction.h:132-143)
        const Dual f = scaledJacobi(i, 0, 0, 2.0 * xi - one + eta + zeta, one - eta - zeta) *
                       scaledJacobi(j, 2 * i + 1, 0, 2.0 * eta - one + zeta, one - zeta) *
                       scaledJacobi(k, 2 * i + 2 * j + 2, 0, 2.0 * zeta - one, one);
        phi[l] = f.v;
        for (int x = 0; x < 3; ++x)
          dphi[x * B + l] = f.d[0] * grad[0][x] + f.d[1] * grad[1][x] + f.d[2] * grad[2][x];
        ++l;
      }
}

// Cell containing each point (lowest id among the cells that contain it, barycentric coordinates
// >= -tol), found through a uniform grid of cell bounding boxes; -1 outside the mesh.  xez gets
// the reference coordinates (Numerical/Transformation.cpp:47-64).
void locatePoints(const HostMesh& m, int64_t np, const double* xyz, std::vector<int64_t>& cell,
                  std::vector<double>& xez) {
  cell.assign(np, -1);
  xez.assign(np * 3, 0.0);
  if (m.n == 0 || np == 0) return;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (size_t i = 0; i < m.coords.size(); i += 3)
    for (int x = 0; x < 3; ++x) {
      lo[x] = std::min(lo[x], m.coords[i + x]);
      hi[x] = std::max(hi[x], m.coords[i + x]);
    }
  const int g = std::max(1, std::min(256, (int)std::cbrt((double)m.n / 4.0)));
  double h[3];
  for (int x = 0; x < 3; ++x) h[x] = (hi[x] - lo[x]) / g + 1e-300;
  auto bin = [&](double v, int x) { return std::max(0, std::min(g - 1, (int)((v - lo[x]) / h[x]))); };
  std::vector<std::vector<int64_t>> grid((size_t)g * g * g);
  for (int64_t c = 0; c < m.n; ++c) {
    int b0[3], b1[3];
    for (int x = 0; x < 3; ++x) {
      double a = 1e300, b = -1e300;
      for (int k = 0; k < 4; ++k) {
        a = std::min(a, m.coords[c * 12 + k * 3 + x]);
        b = std::max(b, m.coords[c * 12 + k * 3 + x]);
      }
      b0[x] = bin(a, x);
      b1[x] = bin(b, x);
    }
    for (int i = b0[0]; i <= b1[0]; ++i)
      for (int j = b0[1]; j <= b1[1]; ++j)
        for (int k = b0[2]; k <= b1[2]; ++k) grid[((size_t)k * g + j) * g + i].push_back(c);
  }
  for (int64_t p = 0; p < np; ++p) {
    const double* q = xyz + p * 3;
    bool inside = true;
    for (int x = 0; x < 3; ++x) inside = inside && q[x] >= lo[x] - 1e-9 * (hi[x] - lo[x]) && q[x] <= hi[x] + 1e-9 * (hi[x] - lo[x]);
    if (!inside) continue;
    const auto& list = grid[((size_t)bin(q[2], 2) * g + bin(q[1], 1)) * g + bin(q[0], 0)];
    for (int64_t c : list) {
      const double* v = &m.coords[c * 12];
      // solve [v1-v0 v2-v0 v3-v0] (xi, eta, zeta) = q - v0 (Cramer)
      double a[3][3], r[3];
      for (int x = 0; x < 3; ++x) {
        for (int k = 0; k < 3; ++k) a[x][k] = v[(k + 1) * 3 + x] - v[x];
        r[x] = q[x] - v[x];
      }
      const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
      double s[3];
      for (int k = 0; k < 3; ++k) {
        double b[3][3];
        for (int x = 0; x < 3; ++x)
          for (int y = 0; y < 3; ++y) b[x][y] = y == k ? r[x] : a[x][y];
        s[k] = (b[0][0] * (b[1][1] * b[2][2] - b[1][2] * b[2][1]) - b[0][1] * (b[1][0] * b[2][2] - b[1][2] * b[2][0]) +
                b[0][2] * (b[1][0] * b[2][1] - b[1][1] * b[2][0])) / det;
      }
      const double tol = 1e-10;
      if (s[0] >= -tol && s[1] >= -tol && s[2] >= -tol && s[0] + s[1] + s[2] <= 1 + tol) {
        if (cell[p] < 0 || c < cell[p]) {
          cell[p] = c;
          for (int k = 0; k < 3; ++k) xez[p * 3 + k] = s[k];
        }
      }
    }
  }
}

}  // namespace sei
