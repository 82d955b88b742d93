// Device helpers shared by the generated ADER-DG kernels.
#pragma once
#include <cstddef>

// Taylor coefficients of one time integration, passed by value (up to order 8).
struct SeiCoeffs {
  float c[8];
};

// Relaxation frequencies of the viscoelastic mechanisms (kernel argument).
struct SeiOmega {
  float w[3];
};

// Column of N floats starting at a 16-byte aligned address (N % 4 == 0) or any address.
template <int N>
__device__ __forceinline__ void sei_load_col(const float* __restrict__ p, float (&v)[N]) {
  if constexpr (N % 4 == 0) {
    const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
      const float4 t = __ldg(p4 + i);
      v[4 * i] = t.x;
      v[4 * i + 1] = t.y;
      v[4 * i + 2] = t.z;
      v[4 * i + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = __ldg(p + i);
  }
}

template <int N, int M>
__device__ __forceinline__ void sei_store_col(float* __restrict__ p, const float (&v)[M]) {
  static_assert(N <= M, "store longer than array");
  if constexpr (N % 4 == 0) {
    float4* p4 = reinterpret_cast<float4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) p4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = v[i];
  }
}

// Scalar stores for packed layouts without 16-byte alignment.
template <int N, int M>
__device__ __forceinline__ void sei_store_col_scalar(float* __restrict__ p, const float (&v)[M]) {
  static_assert(N <= M, "store longer than array");
#pragma unroll
  for (int i = 0; i < N; ++i) p[i] = v[i];
}

// Asynchronous 16-byte global -> shared copies (both addresses 16-byte aligned).
__device__ __forceinline__ void sei_cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void sei_cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void sei_cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Face traces of the local-integral kernel, staged in shared memory after the trace exchange
// buffer of the flux stage ([9][R][32] floats, R = the template argument B):
// the row of (cell lane, quantity q) holds FP floats (zero padded); a cell's 9 rows are followed
// by 4 floats of padding, so 16-byte writes of a quarter warp (8 cells) hit distinct banks.
template <int FP>
constexpr int seiTraceStageStride() { return 9 * FP + 4; }

template <int B, int F, int FP>
__device__ __forceinline__ void sei_stage_trace(float* sm, int lane, int q, const float (&T)[F]) {
  float4* st = reinterpret_cast<float4*>(sm + 9 * B * 32 + lane * seiTraceStageStride<FP>() + q * FP);
#pragma unroll
  for (int m4 = 0; m4 < FP / 4; ++m4) {
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = 4 * m4 + u < F ? T[4 * m4 + u < F ? 4 * m4 + u : 0] : 0.f;
    st[m4] = make_float4(v[0], v[1], v[2], v[3]);
  }
}

// Coalesced 16-byte store of the staged face-f traces of a CPB-cell block to
// trace[4][plane][9][FP] (n cells in this launch, plane cells per face plane).
// Not unrolled: the generated kernels are large and their instruction cache is the limit.
template <int B, int F, int FP, int CPB>
__device__ __forceinline__ void sei_store_traces(int n, const float* sm, float* trace, int f, int plane) {
  constexpr int R4 = 9 * FP / 4;  // float4 per cell
  const float* st = sm + 9 * B * 32;
  const int cell0 = blockIdx.x * CPB;
  float4* dst = reinterpret_cast<float4*>(trace + ((size_t)f * plane + cell0) * 9 * FP);
#pragma unroll 1
  for (int idx = threadIdx.x; idx < CPB * R4; idx += blockDim.x) {
    const int L = idx / R4, rem = idx - L * R4;
    if (cell0 + L < n) dst[idx] = *reinterpret_cast<const float4*>(st + L * seiTraceStageStride<FP>() + 4 * rem);
  }
}
