// Launchers of the viscoelastic CUDA-core kernels for one convergence order.  Included by
// kernels_visco_o{4,5}.cu after the generated kernel bodies (seissol_gb300/codegen/gen_visco.py)
// with SEI_VORDER defined.
#pragma once
#include <cuda_runtime.h>

#include "internal.h"

#define SEI_VCAT2(a, b) a##b
#define SEI_VCAT(a, b) SEI_VCAT2(a, b)

namespace {
namespace KV = SEI_VCAT(sei_v, SEI_VORDER);


SeiOmega toOmega(const sei::ViscoArrays& d) {
  SeiOmega o{};
  for (int i = 0; i < 3; ++i) o.w[i] = d.omega[i];
  return o;
}

int launchVAder(const sei::ViscoArrays& d, const float* coeffs, void* stream) {
  if (d.n <= 0) return 0;
  // kWA cells per CTA, 15 column tasks of kWA threads: X, M and IM of kWA cells
  const size_t smem = sizeof(float) * (9 + 36) * KV::kB * KV::kWA;
  if (cudaFuncSetAttribute(KV::SEI_VCAT(sei_vader_o, SEI_VORDER), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  SeiCoeffs c{};
  for (int i = 0; i < KV::kOrder; ++i) c.c[i] = coeffs[i];
  const int blocks = (d.n + KV::kWA - 1) / KV::kWA;
  KV::SEI_VCAT(sei_vader_o, SEI_VORDER)<<<blocks, 15 * KV::kWA, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.star_nz, d.grad, d.theta, toOmega(d), c, d.derivs, d.dslot);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchVLint(const sei::ViscoArrays& d, void* stream) {
  if (d.n <= 0) return 0;
  // 16 cells per CTA, 15 column tasks of 16 threads: the exchange X and the theta sums TH of 16 cells
  const size_t smem = sizeof(float) * 18 * KV::kB * KV::kCPBA;
  if (cudaFuncSetAttribute(KV::SEI_VCAT(sei_vlint_o, SEI_VORDER), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  const int blocks = (d.n + KV::kCPBA - 1) / KV::kCPBA;
  KV::SEI_VCAT(sei_vlint_o, SEI_VORDER)<<<blocks, 15 * KV::kCPBA, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.star_nz, d.grad, d.theta, toOmega(d), d.aplus, d.wplus, d.ftype);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchVNeighbor(const sei::ViscoArrays& d, void* stream) {
  if (d.n <= 0) return 0;
  const size_t smem = sizeof(float) * 9 * KV::kF * KV::kCPBA;
  const int blocks = (d.n + KV::kCPBA - 1) / KV::kCPBA;
  KV::SEI_VCAT(sei_vneighbor_o, SEI_VORDER)<<<blocks, 15 * KV::kCPBA, smem, (cudaStream_t)stream>>>(
      d.n, d.Q, d.I, d.aminus, d.wminus, d.nbr, d.rel, d.ftype, toOmega(d));
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
}  // namespace

namespace sei {
ViscoKernels SEI_VCAT(viscoKernels, SEI_VORDER)() {
  return ViscoKernels{launchVAder, launchVLint, launchVNeighbor, KV::kDerivSize};
}
}  // namespace sei
