// Integration buffers of local time stepping: a cell with a coarser neighbour sums its
// time-integrated DOFs over the sub-steps that make up one step of that neighbour
// (reference: the buffers of src/Solver/TimeStepping/TimeCluster.cpp, read by
// TimeCommon::computeIntegrals, src/Kernels/TimeCommon.cpp:40-87).
#include <cuda_runtime.h>

#include "internal.h"

namespace {

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

}  // namespace

namespace sei {

int launchLtsBuffer(int m, const int32_t* cell, const int32_t* dst, float* pool, int blk, int reset, void* stream) {
  if (m <= 0) return 0;
  if (blk % 4) return -1;
  const int blk4 = blk / 4;
  const long threads = (long)m * blk4;
  sei_lts_buffer<<<(int)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(m, cell, dst, pool, blk4, reset);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sei
