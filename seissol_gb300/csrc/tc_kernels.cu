// Tensor-core (tcgen05) kernels of the element update, mixed precision.
//
// Volume + local flux (Local::computeIntegral, codegen/kernels/aderdg.py:337-386) of a tile of
// 14 cells.  The 128 TMEM lanes are the rows (cell, quantity) = 9 c + q (rows 126, 127 unused).
//   MMA 1:  D1[r, n] = sum_l I[r, l] V[n, l],  V = [kDivM_0; kDivM_1; kDivM_2; fMrT_0..3]
//   CUDA:   vol[(c,p), k] = sum_e sum_q D1[(c,q), e B + k] star_e[q, p]
//           G[(c,p), f F + m] = sum_q D1[(c,q), 3 B + f F + m] AplusT_f[q, p]
//   MMA 2:  D2[r, k] = sum_{f,m} G[r, f F + m] rDivM_f[k, m]
//   Q += vol + D2.
// Products: FP16 split in three terms (x_hi y_hi + x_hi y_lo + x_lo y_hi, FP32 accumulation in
// TMEM) after scaling each data row and each matrix row by a power of two (max |row| in
// [0.5, 1)); the matrices arrive pre-split (generated tables) and are staged once per
// persistent CTA by bulk TMA.  Per-cell 9x9 mixing exchanges rows through shared memory.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"
#include "_gen/tc_tables_o4.cuh"
#include "_gen/tc_tables_o5.cuh"
#include "_gen/tc_tables_o6.cuh"
#include "_gen/tc_nb_o4.cuh"
#include "_gen/tc_nb_o5.cuh"
#include "_gen/tc_nb_o6.cuh"

namespace {

constexpr uint32_t kMaxPolls = 1u << 26;
constexpr int kCellsPerTile = 14;

// Non-zero pattern of the elastic star matrix: sources q of output column p, index into the
// 24 stored non-zeros (-1: none), as in the CUDA-core kernels.
__constant__ int c_tsrc[9][3] = {{6, 7, 8}, {6, 7, 8}, {6, 7, 8}, {6, 7, 6}, {7, 8, 7}, {6, 8, 6}, {0, 3, 5}, {1, 3, 4}, {2, 4, 5}};
__constant__ int c_tnzi[9][3] = {{0, 1, 2}, {3, 4, 5}, {6, 7, 8}, {9, 10, -1}, {11, 12, -1}, {13, 14, -1}, {15, 16, 17}, {18, 19, 20}, {21, 22, 23}};

template <int ORD>
struct Dims {
  static constexpr int B = ORD * (ORD + 1) * (ORD + 2) / 6;
  static constexpr int Bp = (B + 3) / 4 * 4;
  static constexpr int F = ORD * (ORD + 1) / 2;
  static constexpr int KB = (B + 15) / 16 * 16;
  static constexpr int N1 = (3 * B + 4 * F + 15) / 16 * 16;
  static constexpr int K2 = (4 * F + 15) / 16 * 16;
  static constexpr int N2 = (B + 15) / 16 * 16;
  static constexpr int KA = KB > K2 ? KB : K2;
  static constexpr int XC = B > 4 * F ? B : 4 * F;
  static constexpr uint32_t kCols = N1 <= 32 ? 32 : (N1 <= 64 ? 64 : (N1 <= 128 ? 128 : 256));
  static constexpr size_t kOpVol = (size_t)N1 * KB * 4;  // hi + lo, bytes
  static constexpr size_t kOpRd = (size_t)N2 * K2 * 4;
  static constexpr size_t kA = (size_t)128 * KA * 4;   // hi + lo halves
  static constexpr size_t kX = (size_t)XC * 128 * 4;
  static constexpr size_t kSmem = kOpVol + kOpRd + kA + kX;
  static_assert(N1 <= 256 && N2 <= 256, "MMA N limit");
};

template <int N>
__device__ __forceinline__ int rowExp(const float (&v)[N], int n) {
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < N; ++k)
    if (k < n) m = fmaxf(m, fabsf(v[k]));
  int e = 0;
  (void)frexpf(m, &e);
  return m > 0.f ? e : 0;
}

// Writes v[0..n) * 2^-e as FP16 hi and lo parts into row r of the A operand (K capacity ka).
template <int KP, int N>
__device__ __forceinline__ void writeRow(__half* aHi, __half* aLo, int r, const float (&v)[N], int e, int n, int ka) {
#pragma unroll
  for (int j = 0; j < KP / 8; ++j) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k0 = 8 * j + 2 * i, k1 = k0 + 1;
      const float x0 = (k0 < n && k0 < N) ? ldexpf(v[k0 < N ? k0 : 0], -e) : 0.f;
      const float x1 = (k1 < n && k1 < N) ? ldexpf(v[k1 < N ? k1 : 0], -e) : 0.f;
      const __half h0 = __float2half_rn(x0), h1 = __float2half_rn(x1);
      const __half l0 = __float2half_rn(x0 - __half2float(h0)), l1 = __float2half_rn(x1 - __half2float(h1));
      h[i] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
      l[i] = (uint32_t)__half_as_ushort(l0) | ((uint32_t)__half_as_ushort(l1) << 16);
    }
    const uint32_t off = sei_tc::kmajorOffset16(r, 8 * j, ka / 8) / 2;
    *reinterpret_cast<uint4*>(aHi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(aLo + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// Issues the three split products over ksteps K steps of 16: D (+)= A B^T, then commits.
__device__ __forceinline__ void issueSplit(uint32_t d, const __half* aHi, const __half* aLo, int ka,
                                           const uint16_t* bHi, const uint16_t* bLo, int kb, int ksteps, uint32_t idesc,
                                           uint64_t* mbar) {
  const uint32_t sboA = (uint32_t)(ka / 8) * 128, sboB = (uint32_t)(kb / 8) * 128;
  const uint32_t pa[3] = {sei_tc::smemAddr(aHi), sei_tc::smemAddr(aHi), sei_tc::smemAddr(aLo)};
  const uint32_t pb[3] = {sei_tc::smemAddr(bHi), sei_tc::smemAddr(bLo), sei_tc::smemAddr(bHi)};
  for (int s = 0; s < ksteps; ++s)
#pragma unroll
    for (int t = 0; t < 3; ++t)
      sei_tc::mmaSSf16(d, sei_tc::smemDesc(pa[t] + 256 * s, 128, sboA), sei_tc::smemDesc(pb[t] + 256 * s, 128, sboB), idesc,
                       s > 0 || t > 0);
  sei_tc::mmaCommit(mbar);
}

// Calls fn(i, value) for the TMEM columns c0 .. c0+len-1 of this thread's lane, reading
// 16-column chunks aligned to 16 (never past ceil16(c0 + len)).
template <typename Fn>
__device__ __forceinline__ void forColumns(uint32_t tbase, int c0, int len, Fn&& fn) {
  const int first = c0 & ~15;
  for (int cc = first; cc < c0 + len; cc += 16) {
    float v[16];
    sei_tc::tmemLoad16(tbase + (uint32_t)cc, v);
    sei_tc::tmemLoadWait();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int col = cc + i;
      if (col >= c0 && col < c0 + len) fn(col - c0, v[i]);
    }
  }
}

// acc[k] += column k * scale * sc[k] for k < LEN (compile-time indices; reads ceil16(LEN) columns).
template <int LEN, int N>
__device__ __forceinline__ void accumulateColumns(uint32_t tbase, float (&acc)[N], float scale, const float* sc) {
#pragma unroll
  for (int cc = 0; cc < LEN; cc += 16) {
    float v[16];
    sei_tc::tmemLoad16(tbase + (uint32_t)cc, v);
    sei_tc::tmemLoadWait();
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (cc + i < LEN && cc + i < N) acc[cc + i < N ? cc + i : 0] += v[i] * scale * __ldg(sc + cc + i);
  }
}

template <int ORD>
__global__ void __launch_bounds__(128, 1) sei_lint_tc(sei::TcLintArgs A) {
  using D = Dims<ORD>;
  constexpr int B = D::B, Bp = D::Bp, F = D::F;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  uint16_t* opVol = reinterpret_cast<uint16_t*>(sm);
  uint16_t* opRd = reinterpret_cast<uint16_t*>(sm + D::kOpVol);
  __half* aHi = reinterpret_cast<__half*>(sm + D::kOpVol + D::kOpRd);
  __half* aLo = aHi + 128 * D::KA;
  float* X = reinterpret_cast<float*>(sm + D::kOpVol + D::kOpRd + D::kA);
  const int tid = threadIdx.x;
  if (tid < 32) sei_tc::tmemAlloc(&tslot, D::kCols);
  if (tid == 0) {
    sei_tc::mbarInit(&mbar, 1);
    sei_tc::mbarExpectTx(&mbar, (uint32_t)(D::kOpVol + D::kOpRd));
    sei_tc::bulkCopyG2S(opVol, A.opVol, (uint32_t)D::kOpVol, &mbar);
    sei_tc::bulkCopyG2S(opRd, A.opRd, (uint32_t)D::kOpRd, &mbar);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot;
  const uint32_t tbase = taddr + ((uint32_t)((tid >> 5) * 32) << 16);
  uint32_t phase = 0;
  bool ok = sei_tc::mbarWait(&mbar, phase, kMaxPolls);
  phase ^= 1;
  const uint16_t* volHi = opVol;
  const uint16_t* volLo = opVol + D::N1 * D::KB;
  const uint16_t* rdHi = opRd;
  const uint16_t* rdLo = opRd + D::N2 * D::K2;
  const int r = tid, q = r % 9;
  const bool rowOk = r < 9 * kCellsPerTile;
  // The padding rows 126 and 127 mix the rows of cell 13: their results are never stored, and
  // every exchange read 9 c + s then stays inside the 128 rows of the buffer.
  const int c = rowOk ? r / 9 : kCellsPerTile - 1;
  const int s0 = c_tsrc[q][0], s1 = c_tsrc[q][1], s2 = c_tsrc[q][2];
  const int ntiles = (A.n + kCellsPerTile - 1) / kCellsPerTile;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int cell = tile * kCellsPerTile + c;
    const bool valid = rowOk && cell < A.n;  // padding rows never store
    const int cl = valid ? cell : 0;
    float st[3][3];
#pragma unroll
    for (int e = 0; e < 3; ++e)
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = c_tnzi[q][s];
        st[e][s] = (valid && i >= 0) ? __ldg(A.star_nz + (size_t)cl * 72 + e * 24 + i) : 0.f;
      }
    float I[Bp], acc[Bp];
    sei_load_col<Bp>(A.I + ((size_t)cl * 9 + q) * Bp, I);
    sei_load_col<Bp>(A.Q + ((size_t)cl * 9 + q) * Bp, acc);
    const int eI = rowExp(I, B);
    writeRow<D::KB>(aHi, aLo, r, I, eI, B, D::KA);
    sei_tc::fenceProxyAsync();
    sei_tc::fenceBeforeSync();
    __syncthreads();
    sei_tc::fenceAfterSync();
    if (tid == 0) issueSplit(taddr, aHi, aLo, D::KA, volHi, volLo, D::KB, D::KB / 16, sei_tc::idescF16(128, D::N1), &mbar);
    ok = sei_tc::mbarWait(&mbar, phase, kMaxPolls) && ok;
    phase ^= 1;
    sei_tc::fenceAfterSync();
    const float sI = ldexpf(1.f, eI);
    // volume, one star matrix at a time
#pragma unroll
    for (int e = 0; e < 3 && !A.traceOnly; ++e) {
      forColumns(tbase, e * B, B, [&](int k, float v) { X[k * 128 + r] = v * sI * __ldg(A.scVol + e * B + k); });
      __syncthreads();
      const float* x0 = X + 9 * c + s0;
      const float* x1 = X + 9 * c + s1;
      const float* x2 = X + 9 * c + s2;
#pragma unroll
      for (int k = 0; k < B; ++k)
        acc[k] += st[e][0] * x0[k * 128] + st[e][1] * x1[k * 128] + st[e][2] * x2[k * 128];
      __syncthreads();
    }
    // face traces -> G = traces . AplusT (per face), the A operand of MMA 2; the traces of
    // every face are also stored for the neighbour kernel of this path
    constexpr int FP = (F + 3) / 4 * 4;
    float* trow = (A.trace && valid) ? A.trace + ((size_t)cell * 9 + q) * FP : nullptr;
    forColumns(tbase, 3 * B, 4 * F, [&](int t, float v) {
      const float x = v * sI * __ldg(A.scVol + 3 * B + t);
      X[t * 128 + r] = x;
      if (trow) trow[(size_t)(t / F) * A.tplane * 9 * FP + t % F] = x;
    });
    if (A.traceOnly) {
      sei_tc::fenceBeforeSync();
      __syncthreads();
      sei_tc::fenceAfterSync();
      continue;
    }
    __syncthreads();
    float G[4 * F];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const bool on = valid && A.ftype[(size_t)cl * 4 + f] != 1;
      float av[9];
#pragma unroll
      for (int s = 0; s < 9; ++s) av[s] = on ? __ldg(A.aplus + ((size_t)cl * 4 + f) * 81 + s + 9 * q) : 0.f;
#pragma unroll
      for (int m = 0; m < F; ++m) {
        float g = 0.f;
#pragma unroll
        for (int s = 0; s < 9; ++s) g = fmaf(X[(f * F + m) * 128 + 9 * c + s], av[s], g);
        G[f * F + m] = g;
      }
    }
    const int eG = rowExp(G, 4 * F);
    writeRow<D::K2>(aHi, aLo, r, G, eG, 4 * F, D::KA);
    sei_tc::fenceProxyAsync();
    sei_tc::fenceBeforeSync();
    __syncthreads();
    sei_tc::fenceAfterSync();
    if (tid == 0) issueSplit(taddr, aHi, aLo, D::KA, rdHi, rdLo, D::K2, D::K2 / 16, sei_tc::idescF16(128, D::N2), &mbar);
    ok = sei_tc::mbarWait(&mbar, phase, kMaxPolls) && ok;
    phase ^= 1;
    sei_tc::fenceAfterSync();
    const float sG = ldexpf(1.f, eG);
    accumulateColumns<B>(tbase, acc, sG, A.scRd);
    if (valid) sei_store_col<Bp>(A.Q + ((size_t)cell * 9 + q) * Bp, acc);
    sei_tc::fenceBeforeSync();
    __syncthreads();
    sei_tc::fenceAfterSync();
  }
  if (!ok && tid == 0) atomicExch(A.status, 1);
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (tid < 32) sei_tc::tmemDealloc(taddr, D::kCols);
}

template <int ORD>
int launchLintTc(const sei::DeviceArrays& d, float* trace, int traceOnly, int* status, int sms, void* stream,
                 const void* opVolSym, const void* scVolSym, const void* opRdSym, const void* scRdSym) {
  using Dm = Dims<ORD>;
  sei::TcLintArgs a{};
  a.trace = trace;
  a.tplane = d.ntotal > 0 ? d.ntotal : d.n;
  a.traceOnly = traceOnly;
  a.n = d.n;
  a.Q = d.Q;
  a.I = d.I;
  a.star_nz = d.star_nz;
  a.aplus = d.aplus;
  a.ftype = d.ftype;
  a.status = status;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, opVolSym) != cudaSuccess) return -1;
  a.opVol = (const uint16_t*)p;
  if (cudaGetSymbolAddress(&p, scVolSym) != cudaSuccess) return -1;
  a.scVol = (const float*)p;
  if (cudaGetSymbolAddress(&p, opRdSym) != cudaSuccess) return -1;
  a.opRd = (const uint16_t*)p;
  if (cudaGetSymbolAddress(&p, scRdSym) != cudaSuccess) return -1;
  a.scRd = (const float*)p;
  if (cudaFuncSetAttribute(sei_lint_tc<ORD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Dm::kSmem) != cudaSuccess)
    return -1;
  const int ntiles = (d.n + kCellsPerTile - 1) / kCellsPerTile;
  const int grid = ntiles < sms ? ntiles : sms;
  if (grid <= 0) return 0;
  sei_lint_tc<ORD><<<grid, 128, Dm::kSmem, (cudaStream_t)stream>>>(a);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// Face-trace map s = fP_h diag(fM)^-1 t of the given order (generated).
template <int ORD, int FP, int F>
__device__ __forceinline__ void applyTraceMap(int h, const float (&t)[FP], float (&s)[F]) {
  if constexpr (ORD == 4) sei_tcnb_o4::applyFp(h, t, s);
  if constexpr (ORD == 5) sei_tcnb_o5::applyFp(h, t, s);
  if constexpr (ORD == 6) sei_tcnb_o6::applyFp(h, t, s);
}

template <int ORD>
struct NbDims {
  static constexpr int B = Dims<ORD>::B, Bp = Dims<ORD>::Bp, F = Dims<ORD>::F;
  static constexpr int FP = (F + 3) / 4 * 4;
  static constexpr int K2 = Dims<ORD>::K2, N2 = Dims<ORD>::N2;
  static constexpr uint32_t kCols = N2 <= 32 ? 32 : (N2 <= 64 ? 64 : 128);
  static constexpr size_t kOp = (size_t)N2 * K2 * 4;       // rDivM stack, hi + lo
  static constexpr size_t kX = (size_t)4 * 128 * FP * 4;   // mapped traces, FP32 [face][row][FP]
  static constexpr size_t kAop = (size_t)128 * K2 * 4;     // A operand, hi + lo (aliases X)
  static constexpr size_t kSmem = kOp + (kX > kAop ? kX : kAop);
};

// Neighbour flux (Neighbor::computeNeighborsIntegral, codegen/kernels/aderdg.py:414-428) of a
// tile of 14 cells from the stored face traces T_f = fMrT_f I of all cells ([face][cell][9][FP]).  Rows of the tile
// are (cell, quantity) = 9 c + q.  For each regular face i with neighbour nb, side j and
// orientation h:
//   thread (c, q):  S_i[q, :] = fP_h diag(fM)^-1 T_j(nb)[q, :]                (CUDA cores, FP32)
//   thread (c, p):  E[(c,p), i F + m] = sum_q AminusT_i[q, p] S_i[q, m]      (CUDA cores, FP32)
//   MMA:            D[(c,p), k] = sum_{i,m} E[(c,p), i F + m] rDivM_i[k, m]  (split FP16 x3)
//   Q += D.
// Three 128-thread CTAs per SM (74 KB of shared memory each at order 6) overlap one another's
// waits; the E operand aliases the exchange buffer of the mapped traces.
template <int ORD>
__global__ void __launch_bounds__(128, 3) sei_nb_tc(sei::TcNbArgs A) {
  using D = NbDims<ORD>;
  constexpr int B = D::B, Bp = D::Bp, F = D::F, FP = D::FP, K2 = D::K2, N2 = D::N2;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  uint16_t* opRd = reinterpret_cast<uint16_t*>(sm);
  float* X = reinterpret_cast<float*>(sm + D::kOp);
  __half* aHi = reinterpret_cast<__half*>(sm + D::kOp);
  __half* aLo = aHi + 128 * K2;
  const int tid = threadIdx.x;
  if (tid < 32) sei_tc::tmemAlloc(&tslot, D::kCols);
  if (tid == 0) {
    sei_tc::mbarInit(&mbar, 1);
    sei_tc::mbarExpectTx(&mbar, (uint32_t)D::kOp);
    sei_tc::bulkCopyG2S(opRd, A.opRd, (uint32_t)D::kOp, &mbar);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot;
  const uint32_t tbase = taddr + ((uint32_t)((tid >> 5) * 32) << 16);
  uint32_t phase = 0;
  bool ok = sei_tc::mbarWait(&mbar, phase, kMaxPolls);
  phase ^= 1;
  const uint16_t* rdHi = opRd;
  const uint16_t* rdLo = opRd + N2 * K2;
  const int r = tid, q = r % 9;
  const bool rowOk = r < 9 * kCellsPerTile;
  // Padding rows 126, 127 compute with cell 13 and never store.
  const int c = rowOk ? r / 9 : kCellsPerTile - 1;
  const int ntiles = (A.n + kCellsPerTile - 1) / kCellsPerTile;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int cell = tile * kCellsPerTile + c;
    const bool valid = rowOk && cell < A.n;
    const int cl = cell < A.n ? cell : A.n - 1;
    // L2 prefetch of the next tile of this CTA: its DOFs and AminusT (contiguous), then, once
    // the neighbour indices have arrived, the trace rows its faces read
    const int nt = tile + (int)gridDim.x;
    int pfNb = -1, pfRl = 0;
    if (nt < ntiles) {
      const int c0 = nt * kCellsPerTile;
      const int cnt = A.n - c0 < kCellsPerTile ? A.n - c0 : kCellsPerTile;
      if (tid == 0) {
        sei_tc::prefetchL2(A.Q + (size_t)c0 * 9 * Bp, (uint32_t)(cnt * 9 * Bp * 4));
        sei_tc::prefetchL2(A.aminus + (size_t)c0 * 4 * 81, (uint32_t)(cnt * 4 * 81 * 4));
      }
      if (tid < 4 * cnt) {
        const size_t f = (size_t)c0 * 4 + tid;
        pfNb = A.ftype[f] == 0 ? __ldg(A.nbr + f) : -1;
        pfRl = A.rel[f];
      }
    }
    bool on[4];
    // (1) thread (c, q): the raw trace rows of the four faces arrive together by cp.async into
    // this thread's rows of X, AminusT into registers meanwhile; then the map fP_h diag(fM)^-1
    // in place (each thread touches only its own rows until the barrier)
    int hs[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int nb = __ldg(A.nbr + (size_t)cl * 4 + i);
      const int rl = A.rel[(size_t)cl * 4 + i];
      on[i] = cell < A.n && nb >= 0 && nb < A.ntotal && A.ftype[(size_t)cl * 4 + i] == 0;
      hs[i] = rl >> 2;
      float* xr = X + ((size_t)i * 128 + r) * FP;
      if (on[i]) {
        const float* src = A.trace + (((size_t)(rl & 3) * A.ntotal + nb) * 9 + q) * FP;
#pragma unroll
        for (int m4 = 0; m4 < FP / 4; ++m4) sei_cp_async16(xr + 4 * m4, src + 4 * m4);
      }
    }
    sei_cp_async_commit();
    float av[4][9];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float* am = A.aminus + ((size_t)cl * 4 + i) * 81 + 9 * q;
#pragma unroll
      for (int s2 = 0; s2 < 9; ++s2) av[i][s2] = on[i] ? __ldg(am + s2) : 0.f;
    }
    sei_cp_async_wait<0>();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float4* xr = reinterpret_cast<float4*>(X + ((size_t)i * 128 + r) * FP);
      float s[F];
      if (on[i]) {
        float t[FP];
#pragma unroll
        for (int m4 = 0; m4 < FP / 4; ++m4) {
          const float4 v = xr[m4];
          t[4 * m4] = v.x;
          t[4 * m4 + 1] = v.y;
          t[4 * m4 + 2] = v.z;
          t[4 * m4 + 3] = v.w;
        }
        applyTraceMap<ORD>(hs[i], t, s);
      } else {
#pragma unroll
        for (int m = 0; m < F; ++m) s[m] = 0.f;
      }
#pragma unroll
      for (int m4 = 0; m4 < FP / 4; ++m4)
        xr[m4] = make_float4(4 * m4 < F ? s[4 * m4 < F ? 4 * m4 : 0] : 0.f,
                             4 * m4 + 1 < F ? s[4 * m4 + 1 < F ? 4 * m4 + 1 : 0] : 0.f,
                             4 * m4 + 2 < F ? s[4 * m4 + 2 < F ? 4 * m4 + 2 : 0] : 0.f,
                             4 * m4 + 3 < F ? s[4 * m4 + 3 < F ? 4 * m4 + 3 : 0] : 0.f);
    }
    __syncthreads();
    // (2) thread (c, p = q): E row = sum_q AminusT_i[q, p] S_i[q, :] over the faces
    float E[4 * F];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int m = 0; m < F; ++m) E[i * F + m] = 0.f;
#pragma unroll
      for (int s2 = 0; s2 < 9; ++s2) {
        const float4* xs = reinterpret_cast<const float4*>(X + ((size_t)i * 128 + 9 * c + s2) * FP);
#pragma unroll
        for (int m4 = 0; m4 < FP / 4; ++m4) {
          const float4 x = xs[m4];
          const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (4 * m4 + u < F) E[i * F + 4 * m4 + u] = fmaf(xv[u], av[i][s2], E[i * F + 4 * m4 + u]);
        }
      }
    }
    __syncthreads();  // every read of X precedes the A operand that overwrites it
    const int eE = rowExp(E, 4 * F);
    writeRow<K2>(aHi, aLo, r, E, eE, 4 * F, K2);
    sei_tc::fenceProxyAsync();
    sei_tc::fenceBeforeSync();
    __syncthreads();
    sei_tc::fenceAfterSync();
    if (tid == 0) issueSplit(taddr, aHi, aLo, K2, rdHi, rdLo, K2, K2 / 16, sei_tc::idescF16(128, N2), &mbar);
    if (pfNb >= 0 && pfNb < A.ntotal)
      sei_tc::prefetchL2(A.trace + ((size_t)(pfRl & 3) * A.ntotal + pfNb) * 9 * FP, (uint32_t)(9 * FP * 4));
    float acc[Bp];
    sei_load_col<Bp>(A.Q + ((size_t)cl * 9 + q) * Bp, acc);
    ok = sei_tc::mbarWait(&mbar, phase, kMaxPolls) && ok;
    phase ^= 1;
    sei_tc::fenceAfterSync();
    accumulateColumns<B>(tbase, acc, ldexpf(1.f, eE), A.scRd);
    if (valid) sei_store_col<Bp>(A.Q + ((size_t)cell * 9 + q) * Bp, acc);
    sei_tc::fenceBeforeSync();
    __syncthreads();
    sei_tc::fenceAfterSync();
  }
  if (!ok && tid == 0) atomicExch(A.status, 1);
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (tid < 32) sei_tc::tmemDealloc(taddr, D::kCols);
}

template <int ORD>
int launchNbTc(const sei::DeviceArrays& d, const float* trace, int* status, int sms, int ctasPerSm, void* stream,
               const void* opRdSym, const void* scRdSym) {
  using Dm = NbDims<ORD>;
  sei::TcNbArgs a{};
  a.n = d.n;
  a.ntotal = d.ntotal > 0 ? d.ntotal : d.n;
  a.Q = d.Q;
  a.trace = trace;
  a.aminus = d.aminus;
  a.nbr = d.nbr;
  a.rel = d.rel;
  a.ftype = d.ftype;
  a.status = status;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, opRdSym) != cudaSuccess) return -1;
  a.opRd = (const uint16_t*)p;
  if (cudaGetSymbolAddress(&p, scRdSym) != cudaSuccess) return -1;
  a.scRd = (const float*)p;
  if (cudaFuncSetAttribute(sei_nb_tc<ORD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Dm::kSmem) != cudaSuccess)
    return -1;
  const int ntiles = (d.n + kCellsPerTile - 1) / kCellsPerTile;
  const int perSm = ctasPerSm < 1 ? 1 : (ctasPerSm > 3 ? 3 : ctasPerSm);
  const int grid = ntiles < perSm * sms ? ntiles : perSm * sms;
  if (grid <= 0) return 0;
  sei_nb_tc<ORD><<<grid, 128, Dm::kSmem, (cudaStream_t)stream>>>(a);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

namespace sei {

int launchLintTensorCore(int order, const DeviceArrays& d, float* trace, int traceOnly, int* status, int sms,
                         void* stream) {
  switch (order) {
    case 4:
      return launchLintTc<4>(d, trace, traceOnly, status, sms, stream, (const void*)&sei_tc_o4::kvol_op, (const void*)&sei_tc_o4::kvol_scale,
                                   (const void*)&sei_tc_o4::krdivm_op, (const void*)&sei_tc_o4::krdivm_scale);
    case 5:
      return launchLintTc<5>(d, trace, traceOnly, status, sms, stream, (const void*)&sei_tc_o5::kvol_op, (const void*)&sei_tc_o5::kvol_scale,
                                   (const void*)&sei_tc_o5::krdivm_op, (const void*)&sei_tc_o5::krdivm_scale);
    case 6:
      return launchLintTc<6>(d, trace, traceOnly, status, sms, stream, (const void*)&sei_tc_o6::kvol_op, (const void*)&sei_tc_o6::kvol_scale,
                                   (const void*)&sei_tc_o6::krdivm_op, (const void*)&sei_tc_o6::krdivm_scale);
    default:
      return -1;
  }
}


int launchNeighborTensorCore(int order, const DeviceArrays& d, const float* trace, int* status, int sms, int ctasPerSm,
                             void* stream) {
  switch (order) {
    case 4:
      return launchNbTc<4>(d, trace, status, sms, ctasPerSm, stream, (const void*)&sei_tc_o4::krdivm_op,
                           (const void*)&sei_tc_o4::krdivm_scale);
    case 5:
      return launchNbTc<5>(d, trace, status, sms, ctasPerSm, stream, (const void*)&sei_tc_o5::krdivm_op,
                           (const void*)&sei_tc_o5::krdivm_scale);
    case 6:
      return launchNbTc<6>(d, trace, status, sms, ctasPerSm, stream, (const void*)&sei_tc_o6::krdivm_op,
                           (const void*)&sei_tc_o6::krdivm_scale);
    default:
      return -1;
  }
}

}  // namespace sei
