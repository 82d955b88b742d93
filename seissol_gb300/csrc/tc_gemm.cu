// Single-tile tensor-core GEMM D = A B^T (A: 128 x K, B: N x K, row-major floats) on tcgen05
// kind::tf32 with TMEM accumulator: the self-check of the descriptor and TMEM conventions used
// by the element-update kernels.  terms = 1: plain TF32; terms = 3: split TF32
// (A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32 accumulation).
#include <cuda_runtime.h>

#include "internal.h"
#include "tc.cuh"

namespace {

constexpr uint32_t kMaxPolls = 1u << 24;

__global__ void __launch_bounds__(128) sei_tc_gemm_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                           float* __restrict__ D, int N, int K, int terms,
                                                           int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int kc = K / 4;
  float* aHi = reinterpret_cast<float*>(smem);
  float* aLo = aHi + 128 * K;
  float* bHi = aLo + 128 * K;
  float* bLo = bHi + N * K;
  const int tid = threadIdx.x;
  uint32_t ncols = 32;
  while (ncols < (uint32_t)N) ncols <<= 1;
  if (tid < 32) sei_tc::tmemAlloc(&tslot, ncols);
  if (tid == 0) sei_tc::mbarInit(&mbar, 1);
  // operands: thread tid owns row tid of A and rows tid, tid + 128 of B
  for (int k = 0; k < K; ++k) {
    float hi, lo;
    sei_tc::splitTf32(A[tid * K + k], hi, lo);
    const uint32_t o = sei_tc::kmajorOffset(tid, k, kc) / 4;
    aHi[o] = hi;
    aLo[o] = lo;
  }
  for (int r = tid; r < N; r += 128)
    for (int k = 0; k < K; ++k) {
      float hi, lo;
      sei_tc::splitTf32(B[r * K + k], hi, lo);
      const uint32_t o = sei_tc::kmajorOffset(r, k, kc) / 4;
      bHi[o] = hi;
      bLo[o] = lo;
    }
  sei_tc::fenceProxyAsync();
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    const uint32_t idesc = sei_tc::idescTf32(128, N);
    const uint32_t sbo = (uint32_t)kc * 128;
    const uint32_t pa[3] = {sei_tc::smemAddr(aHi), sei_tc::smemAddr(aHi), sei_tc::smemAddr(aLo)};
    const uint32_t pb[3] = {sei_tc::smemAddr(bHi), sei_tc::smemAddr(bLo), sei_tc::smemAddr(bHi)};
    for (int s = 0; s < K / 8; ++s)
      for (int t = 0; t < terms; ++t)
        sei_tc::mmaSS(taddr, sei_tc::smemDesc(pa[t] + 256 * s, 128, sbo), sei_tc::smemDesc(pb[t] + 256 * s, 128, sbo),
                      idesc, s > 0 || t > 0);
    sei_tc::mmaCommit(&mbar);
  }
  const bool ok = sei_tc::mbarWait(&mbar, 0, kMaxPolls);
  if (!ok && tid == 0) atomicExch(status, 1);
  sei_tc::fenceAfterSync();
  if (ok) {
    const uint32_t lane_base = (uint32_t)((tid >> 5) * 32) << 16;
    for (int c = 0; c < N; c += 16) {
      float v[16];
      sei_tc::tmemLoad16(taddr + lane_base + (uint32_t)c, v);
      sei_tc::tmemLoadWait();
#pragma unroll
      for (int i = 0; i < 16; ++i) D[tid * N + c + i] = v[i];
    }
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (tid < 32) sei_tc::tmemDealloc(taddr, ncols);
}

}  // namespace

extern "C" int sei_tc_gemm_check(const float* A, const float* B, float* D, int N, int K, int terms) {
  if (!A || !B || !D || N < 16 || N > 256 || N % 16 || K < 8 || K > 64 || K % 8 || (terms != 1 && terms != 3))
    return SEI_ERR_ARG;
  const size_t smem = sizeof(float) * (size_t)(2 * 128 * K + 2 * N * K);
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dS = nullptr;
  int rc = SEI_OK, st = 0;
  if (cudaMalloc(&dA, 128 * K * 4) || cudaMalloc(&dB, N * K * 4) || cudaMalloc(&dD, 128 * N * 4) || cudaMalloc(&dS, 4)) {
    rc = SEI_ERR_OOM;
  } else if (cudaMemcpy(dA, A, 128 * K * 4, cudaMemcpyHostToDevice) || cudaMemcpy(dB, B, N * K * 4, cudaMemcpyHostToDevice) ||
             cudaMemset(dS, 0, 4) ||
             cudaFuncSetAttribute(sei_tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) {
    rc = SEI_ERR_CUDA;
  } else {
    sei_tc_gemm_kernel<<<1, 128, smem>>>(dA, dB, dD, N, K, terms, dS);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(D, dD, 128 * N * 4, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost))
      rc = SEI_ERR_CUDA;
    else if (st)
      rc = SEI_ERR_TIMEOUT;
  }
  cudaGetLastError();
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dS);
  return rc;
}
