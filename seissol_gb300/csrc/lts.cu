// Integration buffers of local time stepping: a cell with a coarser neighbour sums its
// time-integrated DOFs over the sub-steps that make up one step of that neighbour
// (reference: the buffers of src/Solver/TimeStepping/TimeCluster.cpp, read by
// TimeCommon::computeIntegrals, src/Kernels/TimeCommon.cpp:40-87).
#include <cuda_runtime.h>

#include "internal.h"

namespace {

struct SeiCoeffsGather {
  float c[8];
};

__global__ void sei_lts_buffer(int m, const int32_t* __restrict__ cell, const int32_t* __restrict__ dst,
                               float* __restrict__ pool, int blk4, int reset) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)m * blk4) return;
  const long e = t / blk4;
  const int j = (int)(t % blk4);
  const float4 v = reinterpret_cast<const float4*>(pool)[(size_t)__ldg(cell + e) * blk4 + j];
  float4* o = reinterpret_cast<float4*>(pool) + (size_t)__ldg(dst + e) * blk4 + j;
  if (reset) {
    *o = v;
  } else {
    float4 w = *o;
    w.x += v.x;
    w.y += v.y;
    w.z += v.z;
    w.w += v.w;
    *o = w;
  }
}

// The buffer of the face traces: trace[f][dst[e]] (=|+=) trace[f][cell[e]] for the four faces f,
// one thread per float4 of a (entry, face) row.
__global__ void sei_lts_trace_buffer(int m, const int32_t* __restrict__ cell, const int32_t* __restrict__ dst,
                                     float* __restrict__ trace, long long plane4, int row4, int reset) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)m * 4 * row4) return;
  const long e = t / (4 * row4);
  const int r = (int)(t - e * 4 * row4);
  const int f = r / row4, j = r - f * row4;
  float4* tr = reinterpret_cast<float4*>(trace) + (size_t)f * plane4;
  const float4 v = tr[(size_t)__ldg(cell + e) * row4 + j];
  float4* o = tr + (size_t)__ldg(dst + e) * row4 + j;
  if (reset) {
    *o = v;
  } else {
    float4 w = *o;
    w.x += v.x;
    w.y += v.y;
    w.z += v.z;
    w.w += v.w;
    *o = w;
  }
}

// One thread per (entry e, quantity q, basis k < bp), consecutive threads along k (coalesced):
// pool[dst[e]][q][k] = sum_i coeffs[i] d[src[e]][i][q][k] for k < b, zero for b <= k < bp
// (Taylor integral of stored full-row derivatives).
__global__ void sei_taylor_gather_full(int m, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                       const float* __restrict__ derivs, int order, int nq, int b, int bp,
                                       SeiCoeffsGather coeffs, float* __restrict__ pool) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long per = (long)nq * bp;
  if (t >= (long)m * per) return;
  const long e = t / per;
  const int r = (int)(t - e * per);
  const int q = r / bp, k = r - q * bp;
  float v = 0.f;
  if (k < b) {
    const float* d = derivs + (size_t)__ldg(src + e) * order * nq * b + (size_t)q * b + k;
    for (int i = 0; i < order; ++i) v = fmaf(coeffs.c[i], __ldg(d + (size_t)i * nq * b), v);
  }
  pool[(size_t)__ldg(dst + e) * per + r] = v;
}

}  // namespace

namespace sei {

int launchTaylorGatherFull(int m, const int32_t* src, const int32_t* dst, const float* derivs, int order, int nq, int b,
                           int bp, const float* coeffs, float* pool, void* stream) {
  if (m <= 0) return 0;
  if (order < 1 || order > 8) return -1;
  SeiCoeffsGather c{};
  for (int i = 0; i < order; ++i) c.c[i] = coeffs[i];
  const long threads = (long)m * nq * bp;
  sei_taylor_gather_full<<<(int)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(m, src, dst, derivs, order, nq,
                                                                                           b, bp, c, pool);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchLtsBuffer(int m, const int32_t* cell, const int32_t* dst, float* pool, int blk, int reset, void* stream) {
  if (m <= 0) return 0;
  if (blk % 4) return -1;
  const int blk4 = blk / 4;
  const long threads = (long)m * blk4;
  sei_lts_buffer<<<(int)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(m, cell, dst, pool, blk4, reset);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchLtsTraceBuffer(int m, const int32_t* cell, const int32_t* dst, float* trace, int64_t plane, int row,
                         int reset, void* stream) {
  if (m <= 0) return 0;
  if (row % 4) return -1;
  const int row4 = row / 4;
  const long threads = (long)m * 4 * row4;
  sei_lts_trace_buffer<<<(int)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      m, cell, dst, trace, (long long)plane * row4, row4, reset);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sei
