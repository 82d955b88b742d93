// Launchers of the FP32 CUDA-core kernels for one convergence order.  Included by
// kernels_o{4,5,6}.cu after the generated kernel bodies (seissol_gb300/codegen/gen_kernels.py)
// with SEI_ORDER defined.
#pragma once
#include <cuda_runtime.h>

#include "internal.h"
#include "tc.cuh"

#define SEI_CAT2(a, b) a##b
#define SEI_CAT(a, b) SEI_CAT2(a, b)

namespace {
namespace K = SEI_CAT(sei_o, SEI_ORDER);

SeiCoeffs toCoeffs(const float* c) {
  SeiCoeffs s{};
  for (int i = 0; i < K::kOrder; ++i) s.c[i] = c[i];
  return s;
}

int launchLocal(const sei::DeviceArrays& d, const float* coeffs, void* stream) {
  if (d.n <= 0) return 0;
  const size_t smem = sizeof(float) * 9 * K::kB * 32;
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_local_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  K::SEI_CAT(sei_local_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.star_nz, d.aplus, d.ftype, toCoeffs(coeffs), d.derivs, d.dslot);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchNeighbor(const sei::DeviceArrays& d, void* stream) {
  if (d.n <= 0) return 0;
  const size_t smem = sizeof(float) * 9 * K::kF * 32;
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_neighbor_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  K::SEI_CAT(sei_neighbor_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.aminus, d.nbr, d.rel, d.ftype);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchAder(const sei::DeviceArrays& d, const float* coeffs, void* stream) {
  if (d.n <= 0) return 0;
  // the stage exchange buffer [9][kB][32], also the staging area of the block's DOFs [32][kSt]
  const size_t xs = 9 * K::kB * 32, st = 32 * K::kSt;
  const size_t smem = sizeof(float) * (xs > st ? xs : st);
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_ader_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  K::SEI_CAT(sei_ader_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.star_nz, toCoeffs(coeffs), d.derivs, d.dslot, d.status);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchLint(const sei::DeviceArrays& d, void* stream) {
  if (d.n <= 0) return 0;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  if (d.trace) {
    // the volume stage's exchange buffer, which the flux stage reuses for its trace exchange
    // ([9][kF][32]) followed by the staging rows of the stored face traces
    const size_t vol = 9 * K::kB * 32, flux = 9 * K::kF * 32 + 32 * seiTraceStageStride<K::kFP>();
    const size_t smem = sizeof(float) * (vol > flux ? vol : flux);
    if (cudaFuncSetAttribute(K::SEI_CAT(sei_lint_trace_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    K::SEI_CAT(sei_lint_trace_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
        d.n, d.Q, d.I, d.star_nz, d.aplus, d.ftype, d.trace, d.ntotal > 0 ? d.ntotal : d.n);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
  }
  const size_t smem = sizeof(float) * 9 * K::kB * 32;
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_lint_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  K::SEI_CAT(sei_lint_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(d.n, d.Q, d.I, d.star_nz, d.aplus,
                                                                                d.ftype);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// Volume integral and face traces, no local flux (d.trace required).
int launchLintVol(const sei::DeviceArrays& d, void* stream) {
  if (d.n <= 0) return 0;
  if (!d.trace) return -1;
  // one area: the exchange [9][kB][32], the I staging [32][kSt] and one face's traces [32][kTs]
  const size_t xs = 9 * K::kB * 32, is = 32 * K::kSt, ts = 32 * K::kTs;
  const size_t smem = sizeof(float) * (xs > is ? (xs > ts ? xs : ts) : (is > ts ? is : ts));
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_lintv_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  K::SEI_CAT(sei_lintv_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.star_nz, d.trace, d.ntotal > 0 ? d.ntotal : d.n, d.status);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// ADER + volume + face traces (d.trace required); Q += volume by bulk reduce-adds.
int launchLocalVol(const sei::DeviceArrays& d, const float* coeffs, void* stream) {
  if (d.n <= 0) return 0;
  if (!d.trace) return -1;
  // one area: the exchange [9][kB][32], the DOF staging [32][kSt] and one face's traces [32][kTs]
  const size_t xs = 9 * K::kB * 32, is = 32 * K::kSt, ts = 32 * K::kTs;
  const size_t smem = sizeof(float) * (xs > is ? (xs > ts ? xs : ts) : (is > ts ? is : ts));
  if (cudaFuncSetAttribute(K::SEI_CAT(sei_localv_o, SEI_ORDER), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  const int blocks = (d.n + K::kCPB - 1) / K::kCPB;
  K::SEI_CAT(sei_localv_o, SEI_ORDER)<<<blocks, 288, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.star_nz, toCoeffs(coeffs), d.derivs, d.dslot, d.trace, d.ntotal > 0 ? d.ntotal : d.n, d.status);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchTaylor(int n, const float* derivs, const float* coeffs, float* out, void* stream) {
  if (n <= 0) return 0;
  const long threads = (long)n * 9;
  const int blocks = (int)((threads + 255) / 256);
  K::SEI_CAT(sei_taylor_o, SEI_ORDER)<<<blocks, 256, 0, (cudaStream_t)stream>>>(n, derivs, toCoeffs(coeffs), out);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
int launchTaylorGather(int m, const int32_t* src, const int32_t* dst, const float* derivs, const float* coeffs,
                       float* pool, void* stream) {
  if (m <= 0) return 0;
  const long threads = (long)m * 9;
  const int blocks = (int)((threads + 255) / 256);
  K::SEI_CAT(sei_taylor_gather_o, SEI_ORDER)<<<blocks, 256, 0, (cudaStream_t)stream>>>(m, src, dst, derivs,
                                                                                       toCoeffs(coeffs), pool);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
int launchTraceBlocks(int m, const int32_t* blk, const float* pool, float* trace, int tplane, void* stream) {
  if (m <= 0) return 0;
  const long threads = (long)m * 9;
  K::SEI_CAT(sei_trace_blocks_o, SEI_ORDER)<<<(int)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      m, blk, pool, trace, tplane);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
}  // namespace

namespace sei {
OrderKernels SEI_CAT(orderKernels, SEI_ORDER)() {
  return OrderKernels{launchLocal, launchNeighbor, launchTaylor, launchAder, launchLint, launchTaylorGather,
                      K::kFlopAder, K::kFlopLocal, K::kFlopNeighbor, launchLintVol, launchLocalVol,
                      launchTraceBlocks};
}
}  // namespace sei
