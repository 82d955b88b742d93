// Single-tile tensor-core GEMM D = A B^T (A: 128 x K, B: N x K, row-major floats) on tcgen05
// kind::tf32 with TMEM accumulator: the self-check of the descriptor and TMEM conventions used
// by the element-update kernels.  terms = 1: plain TF32; terms = 3: split TF32
// (A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32 accumulation).
#include <cuda_fp16.h>
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

namespace {

// One M x N x K tile D = A B^T on tcgen05 kind::f16 (FP16 operands, FP32 accumulator) for the
// operand layouts of the element-update kernels: A K-major; B K-major (bMN = 0) or MN-major
// (bMN = 1, core matrix = 8 K rows x 16 bytes of N; N groups contiguous, K groups at stride
// NG * 128; lboIsK selects which descriptor offset holds the K stride).  TMEM is zeroed first and
// all 128 lanes x ceil16(N) columns are returned, so the lane placement of M = 64 results shows.
__global__ void __launch_bounds__(128) sei_tc_layout_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                             float* __restrict__ D, int M, int N, int K, int bMN,
                                                             int lboIsK, int aMN, uint32_t bBytes,
                                                             int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int KC = K / 8, NG = N / 8;
  uint16_t* aT = reinterpret_cast<uint16_t*>(smem);
  uint16_t* bT = reinterpret_cast<uint16_t*>(smem + (size_t)M * K * 2);
  const int tid = threadIdx.x;
  constexpr uint32_t ncols = 256;
  if (tid < 32) sei_tc::tmemAlloc(&tslot, ncols);
  if (tid == 0) sei_tc::mbarInit(&mbar, 1);
  for (uint32_t i = tid; i < bBytes / 2; i += 128) bT[i] = 0;
  __syncthreads();
  const int MG = M / 8;
  for (int i = tid; i < M * K; i += 128) {
    const int r = i / K, k = i % K;
    const uint32_t off = aMN ? (uint32_t)((r >> 3) * 128 + (k >> 3) * MG * 128 + (k & 7) * 16 + (r & 7) * 2)
                             : sei_tc::kmajorOffset16(r, k, KC);
    aT[off / 2] = __half_as_ushort(__float2half_rn(A[i]));
  }
  for (int i = tid; i < N * K; i += 128) {
    const int n = i / K, k = i % K;
    const uint32_t off = bMN ? (uint32_t)((n >> 3) * 128 + (k >> 3) * NG * 128 + (k & 7) * 16 + (n & 7) * 2)
                             : sei_tc::kmajorOffset16(n, k, KC);
    bT[off / 2] = __half_as_ushort(__float2half_rn(B[i]));
  }
  sei_tc::fenceProxyAsync();
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot;
  const uint32_t lane_base = (uint32_t)((tid >> 5) * 32) << 16;
  {
    float z[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) z[i] = 0.f;
    for (uint32_t c = 0; c < ncols; c += 16) sei_tc::tmemStore16(taddr + lane_base + c, z);
    sei_tc::tmemStoreWait();
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  if (tid == 0) {
    const uint32_t idesc = sei_tc::idescF16Major(M, N, aMN, bMN);
    const uint32_t sboA = (uint32_t)KC * 128;
    const uint32_t kStrideB = (uint32_t)NG * 128;
    for (int s = 0; s < K / 16; ++s) {
      const uint32_t kStrideA = (uint32_t)MG * 128;
      const uint64_t ad = aMN ? sei_tc::smemDesc(sei_tc::smemAddr(aT) + 2 * kStrideA * s, kStrideA, 128)
                              : sei_tc::smemDesc(sei_tc::smemAddr(aT) + 256 * s, 128, sboA);
      uint64_t bd;
      if (bMN)
        bd = sei_tc::smemDesc(sei_tc::smemAddr(bT) + 2 * kStrideB * s, lboIsK ? kStrideB : 128, lboIsK ? 128 : kStrideB);
      else
        bd = sei_tc::smemDesc(sei_tc::smemAddr(bT) + 256 * s, 128, sboA);
      sei_tc::mmaSSf16(taddr, ad, bd, idesc, s > 0);
    }
    sei_tc::mmaCommit(&mbar);
  }
  const bool ok = sei_tc::mbarWait(&mbar, 0, kMaxPolls);
  if (!ok && tid == 0) atomicExch(status, 1);
  sei_tc::fenceAfterSync();
  if (ok) {
    const int nc = (N + 15) / 16 * 16;
    for (int c = 0; c < nc; c += 16) {
      float v[16];
      sei_tc::tmemLoad16(taddr + lane_base + (uint32_t)c, v);
      sei_tc::tmemLoadWait();
#pragma unroll
      for (int i = 0; i < 16; ++i) D[tid * nc + c + i] = v[i];
    }
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (tid < 32) sei_tc::tmemDealloc(taddr, ncols);
}

}  // namespace

extern "C" int sei_tc_layout_check(const float* A, const float* B, float* D, int M, int N, int K, int bMN, int lboIsK,
                                   int aMN) {
  if (!A || !B || !D || (M != 64 && M != 128) || N < 8 || N > 128 || N % (M == 64 ? 8 : 16) || K < 16 || K > 96 ||
      K % 16 || (bMN != 0 && bMN != 1) || (aMN != 0 && aMN != 1))
    return SEI_ERR_ARG;
  const int nc = (N + 15) / 16 * 16;
  // B region large enough for either reading of the MN-major strides (all offsets a descriptor can
  // form from N/8 groups and K/8 groups at strides 128 and N/8 * 128 stay inside it).
  const uint32_t ng = (uint32_t)N / 8, kg = (uint32_t)K / 8;
  const uint32_t bBytes = (ng + kg + 2) * (ng + kg + 2) * 128;
  const size_t smem = (size_t)M * K * 2 + bBytes;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dS = nullptr;
  int rc = SEI_OK, st = 0;
  if (cudaMalloc(&dA, (size_t)M * K * 4) || cudaMalloc(&dB, (size_t)N * K * 4) || cudaMalloc(&dD, (size_t)128 * nc * 4) ||
      cudaMalloc(&dS, 4)) {
    rc = SEI_ERR_OOM;
  } else if (cudaMemcpy(dA, A, (size_t)M * K * 4, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dB, B, (size_t)N * K * 4, cudaMemcpyHostToDevice) || cudaMemset(dS, 0, 4) ||
             cudaFuncSetAttribute(sei_tc_layout_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) {
    rc = SEI_ERR_CUDA;
  } else {
    sei_tc_layout_kernel<<<1, 128, smem>>>(dA, dB, dD, M, N, K, bMN, lboIsK, aMN, bBytes, dS);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(D, dD, (size_t)128 * nc * 4, cudaMemcpyDeviceToHost) ||
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

namespace {

// One warp waits on an mbarrier of its own.  arrive = 0: nothing ever arrives on it and nothing
// asynchronous is issued, so the bounded wait gives up after `polls` polls, sets *status and
// returns; arrive = 1: thread 0 arrives first and the wait completes.  The kernels' give-up path,
// exercised without a GPU fault.
__global__ void sei_wait_probe_kernel(uint32_t polls, int arrive, int* __restrict__ status) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) sei_tc::mbarInit(&mbar, 1);
  __syncwarp();
  if (arrive && threadIdx.x == 0)
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(sei_tc::smemAddr(&mbar)) : "memory");
  __syncwarp();
  const bool ok = sei_tc::mbarWait(&mbar, 0, polls);
  if (!ok && threadIdx.x == 0) atomicExch(status, 1);
}

}  // namespace

namespace sei {
int launchWaitProbe(uint32_t polls, int arrive, int* status, void* stream) {
  sei_wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(polls, arrive, status);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
}  // namespace sei

namespace {

// TMEM load-shape check: every thread of a warp writes value = 1000 * lane + column into its own
// lane (columns 0..63, .32x32b stores), then the warp reads the same region back with the shape
// under test and records what each thread received: out[thread][reg] (64 registers at most).
// shape 0: .16x64b.x32 (16 lanes from the warp's quarter base, 32 registers per thread).
__global__ void sei_tc_ld_probe_kernel(int shape, float* __restrict__ out) {
  __shared__ uint32_t tslot;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32) sei_tc::tmemAlloc(&tslot, 64);
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t base = tslot;  // warp 0: lanes 0..31
  for (int c0 = 0; c0 < 64; c0 += 16) {
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = (float)(1000 * lane + c0 + i);
    sei_tc::tmemStore16(base + (uint32_t)c0, v);
  }
  sei_tc::tmemStoreWait();
  __syncwarp();
  uint32_t r[32];
  const uint32_t a = base + (uint32_t)shape;  // shape 0 only (checked by the caller)
  asm volatile(
      "tcgen05.ld.sync.aligned.16x64b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(a)
      : "memory");
  sei_tc::tmemLoadWait();
  if (threadIdx.x < 32)
    for (int i = 0; i < 32; ++i) out[lane * 32 + i] = __uint_as_float(r[i]);
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (threadIdx.x < 32) sei_tc::tmemDealloc(tslot, 64);
}

}  // namespace

extern "C" int sei_tc_ld_probe(int shape, float* out) {
  if (!out || shape != 0) return SEI_ERR_ARG;
  float* d = nullptr;
  int rc = SEI_OK;
  if (cudaMalloc(&d, 32 * 32 * sizeof(float)) != cudaSuccess) return SEI_ERR_OOM;
  sei_tc_ld_probe_kernel<<<1, 32>>>(shape, d);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(out, d, 32 * 32 * sizeof(float), cudaMemcpyDeviceToHost))
    rc = SEI_ERR_CUDA;
  cudaGetLastError();
  cudaFree(d);
  return rc;
}
