// Warm-start network of the rate-and-state Newton solve: 5 -> 64 -> 64 -> 1, tanh, FP32.
//
// Samples are raw (normal stress, absolute shear traction, state variable, a, b, log10 of the
// converged slip rate); the fixed feature and output maps of mlp.cuh turn them into the network's
// inputs and target, each feature shifted and scaled by norm.  Parameters W1[64][5], b1[64],
// W2[64][64], b2[64], W3[64], b3 (4609 floats).  Training minimises the mean squared error of
// the normalised output over the samples the plain Newton solve recorded; Adam updates.
#include <cuda_runtime.h>

#include "internal.h"
#include "mlp.cuh"

namespace {

constexpr int H = sei_mlp::kHidden;
constexpr int kParams = H * 5 + H + H * H + H + H + 1;
constexpr int kChunk = 64;  // samples per block iteration (one per thread)

// Loss and gradient accumulation over samples [0, n): grads += d(loss)/dP with
// loss = sum_s (y_s - t_s)^2 / n.  A block processes chunks of kChunk samples (grid stride,
// one sample per thread); per-sample vectors live in shared memory and every thread owns the
// parameter slice p = t, t + kChunk, ... of the block's gradient (shared), added to the global
// gradient once at the end.
constexpr int kLd = H + 1;
constexpr size_t kGradSmem = sizeof(float) * (2 * (size_t)kParams + kChunk * 5 + 4 * (size_t)kChunk * kLd + kChunk);

__global__ void __launch_bounds__(kChunk) sei_mlp_grad(const float* __restrict__ P, const float* __restrict__ norm,
                                                       const float* __restrict__ X, const float* __restrict__ T, int n,
                                                       float* __restrict__ grads, float* __restrict__ loss) {
  extern __shared__ float dyn[];
  float* sP = dyn;
  float* sG = sP + kParams;
  float* sX = sG + kParams;          // [kChunk][5]
  float* sH1 = sX + kChunk * 5;      // [kChunk][kLd]
  float* sH2 = sH1 + kChunk * kLd;
  float* sD2 = sH2 + kChunk * kLd;
  float* sD1 = sD2 + kChunk * kLd;
  float* sDy = sD1 + kChunk * kLd;   // [kChunk]
  const int t = threadIdx.x;
  for (int i = t; i < kParams; i += kChunk) {
    sP[i] = P[i];
    sG[i] = 0.f;
  }
  __syncthreads();
  const float* W1 = sP;
  const float* b1 = W1 + H * 5;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float b3 = W3[H];
  float lsum = 0.f;
  const float inv_n = 1.f / (float)n;
  float* x = sX + t * 5;
  float* h1 = sH1 + t * kLd;
  float* h2 = sH2 + t * kLd;
  float* d2 = sD2 + t * kLd;
  float* d1 = sD1 + t * kLd;
  for (int base = blockIdx.x * kChunk; base < n; base += gridDim.x * kChunk) {
    const int s = base + t;
    const bool act = s < n;
    double f[5] = {0, 0, 0, 0, 0};
    if (act) {
      const float* r = X + (size_t)s * 5;
      sei_mlp::features(r[0], r[1], r[2], r[3], r[4], f);
    }
    for (int i = 0; i < 5; ++i) x[i] = act ? (float)((f[i] - norm[i]) * norm[5 + i]) : 0.f;
    for (int j = 0; j < H; ++j) {
      float a = b1[j];
      for (int i = 0; i < 5; ++i) a = fmaf(W1[j * 5 + i], x[i], a);
      h1[j] = tanhf(a);
    }
    float y = b3;
    for (int j = 0; j < H; ++j) {
      float a = b2[j];
      for (int i = 0; i < H; ++i) a = fmaf(W2[j * H + i], h1[i], a);
      h2[j] = tanhf(a);
      y = fmaf(W3[j], h2[j], y);
    }
    const float e = act ? y - (float)((sei_mlp::target(f, norm[12], T[s]) - norm[10]) / norm[11]) : 0.f;
    lsum += e * e;
    const float dy = 2.f * e * inv_n;
    sDy[t] = dy;
    for (int j = 0; j < H; ++j) d2[j] = dy * W3[j] * (1.f - h2[j] * h2[j]);
    for (int i = 0; i < H; ++i) {
      float a = 0.f;
      for (int j = 0; j < H; ++j) a = fmaf(W2[j * H + i], d2[j], a);
      d1[i] = a * (1.f - h1[i] * h1[i]);
    }
    __syncthreads();
    for (int p = t; p < kParams; p += kChunk) {
      float acc = 0.f;
      if (p < H * 5) {
        const int j = p / 5, i = p % 5;
        for (int q = 0; q < kChunk; ++q) acc = fmaf(sD1[q * kLd + j], sX[q * 5 + i], acc);
      } else if (p < H * 5 + H) {
        const int j = p - H * 5;
        for (int q = 0; q < kChunk; ++q) acc += sD1[q * kLd + j];
      } else if (p < H * 5 + H + H * H) {
        const int o = p - H * 5 - H, j = o / H, i = o % H;
        for (int q = 0; q < kChunk; ++q) acc = fmaf(sD2[q * kLd + j], sH1[q * kLd + i], acc);
      } else if (p < H * 5 + H + H * H + H) {
        const int j = p - H * 5 - H - H * H;
        for (int q = 0; q < kChunk; ++q) acc += sD2[q * kLd + j];
      } else if (p < kParams - 1) {
        const int j = p - H * 5 - H - H * H - H;
        for (int q = 0; q < kChunk; ++q) acc = fmaf(sDy[q], sH2[q * kLd + j], acc);
      } else {
        for (int q = 0; q < kChunk; ++q) acc += sDy[q];
      }
      sG[p] += acc;
    }
    __syncthreads();
  }
  for (int p = t; p < kParams; p += kChunk) atomicAdd(grads + p, sG[p]);
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((t & 31) == 0) atomicAdd(loss, lsum * inv_n);
}

__global__ void sei_mlp_adam(float* __restrict__ P, const float* __restrict__ grads, float* __restrict__ m,
                             float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float g = grads[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void sei_mlp_predict(const float* __restrict__ P, const float* __restrict__ norm, const float* __restrict__ X,
                                int n, float* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float* W1 = P;
  const float* b1 = W1 + H * 5;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  double f[5];
  sei_mlp::features(X[(size_t)s * 5], X[(size_t)s * 5 + 1], X[(size_t)s * 5 + 2], X[(size_t)s * 5 + 3],
                    X[(size_t)s * 5 + 4], f);
  float x[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) x[i] = (float)((f[i] - norm[i]) * norm[5 + i]);
  float h1[H];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    float a = b1[j];
#pragma unroll
    for (int i = 0; i < 5; ++i) a = fmaf(W1[j * 5 + i], x[i], a);
    h1[j] = tanhf(a);
  }
  float y = W3[H];
#pragma unroll 4
  for (int j = 0; j < H; ++j) {
    float a = b2[j];
#pragma unroll
    for (int i = 0; i < H; ++i) a = fmaf(W2[j * H + i], h1[i], a);
    y = fmaf(W3[j], tanhf(a), y);
  }
  out[s] = (float)(sei_mlp::lnSlipRate(f, norm[12], (double)y * norm[11] + norm[10]) / sei_mlp::kLn10);
}

}  // namespace

namespace sei {

int mlpNumParams() { return kParams; }

int launchMlpGrad(const float* P, const float* norm, const float* X, const float* T, int n, float* grads, float* loss,
                  int sms, void* stream) {
  if (n <= 0) return -1;
  int blocks = (n + kChunk - 1) / kChunk;
  const int cap = sms * 4;
  if (blocks > cap) blocks = cap;
  if (cudaFuncSetAttribute(sei_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem) != cudaSuccess)
    return -1;
  sei_mlp_grad<<<blocks, kChunk, kGradSmem, (cudaStream_t)stream>>>(P, norm, X, T, n, grads, loss);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchMlpAdam(float* P, const float* grads, float* m, float* v, float lr, int step, void* stream) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  sei_mlp_adam<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(P, grads, m, v, lr, b1, b2, 1e-8f, c1, c2);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchMlpPredict(const float* P, const float* norm, const float* X, int n, float* out, void* stream) {
  if (n <= 0) return 0;
  sei_mlp_predict<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(P, norm, X, n, out);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sei
