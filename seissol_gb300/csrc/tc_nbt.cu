// Neighbour flux on the tensor cores in the transposed form (Neighbor::computeNeighborsIntegral,
// codegen/kernels/aderdg.py:414-428), from the face traces T_j = fMrT_j I that the local
// integral of the mixed-precision path stores for every cell and face ([face][cell][9][FP]).
//
// A tile is 8 cells.  The MMA puts the basis index k of the result on the TMEM lanes and the
// tile's (quantity p, cell c) pairs on the 72 columns (n = 8 p + c):
//   D[k, n] = sum_{i, m} rDivM_i[k, m] S_i[m, n],    A = [rDivM_0 | .. | rDivM_3] (64 x 4 KF),
//   S_i[m, (p, c)] = sum_q (fP_h diag(fM)^-1 T_j(nb))[m, q] AminusT_i[q, p]   (FP32, CUDA cores),
// and, when the local flux is fused in (Local.cpp:150-155 shares the lift rDivM_i), also
//   S_i[m, (p, c)] += sum_q T_i(c)[m, q] AplusT_i[q, p]   (the cell's own stored trace),
// so every per-cell 9 x 9 mixing stays inside one thread's registers, and the result lands on
// the lane of the basis function it belongs to: the epilogue adds it to Q with loads and stores
// that are contiguous along the basis index.
//
// A CTA (one per SM) runs four independent tile pipelines, one per warpgroup, over the A table it
// stages once; each warpgroup has its own trace buffer (which its B operand overwrites once the
// mixing has read it), TMEM columns, mbarriers and named barrier, so the four pipelines overlap
// one another's copy and MMA waits.  Per tile and warpgroup:
//   gather  one warp: a bulk copy (cp.async.bulk, mbarrier transaction count) per regular face
//           of the neighbour's trace rows (9 FP floats); L2 prefetch of the tile's DOFs;
//   flux    one thread, on its own mbarrier: the tile's AminusT (and AplusT) rows, one contiguous
//           bulk copy each, issued as soon as the previous tile's mixing has read them;
//   map     thread (face, q), faces ordered by orientation h so a warp mostly runs one branch:
//           the trace row through fP_h diag(fM)^-1 in place (generated literal code);
//   mix     thread (cell c, face i = warp, group of KF / 4 m): S for those m x 9 p in registers
//           (flux matrices from shared memory), all 128 threads busy; per column (p, c) the
//           maximum over all faces and m (warp shuffles, then shared atomics) gives a
//           power-of-two scale; S * 2^-e split into FP16 hi + lo, the B operand (K-major),
//           written over the trace buffer;
//   MMA     one thread: D = A_hi S_hi + A_hi S_lo + A_lo S_hi (FP32 accumulation in TMEM);
//   epilogue  the next tile's gather is issued, then (.16x64b TMEM loads, all 32 threads of a
//           warp) Q[c][p][k] += D[k, (p, c)] 2^{f_k} 2^{e_(p,c)} as f32 reductions performed in L2
//           (one add per element: the result does not depend on their order).
//
// Failure handling: every mbarrier wait is bounded and its outcome made uniform over the
// warpgroup (barrier reduction).  A wait that gives up sets the status word, waits once more
// (bounded) for the copies and MMAs the warpgroup has in flight, and leaves the tile loop; the
// tensor memory is freed after all warpgroups have left.
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
constexpr int kNC = 8;          // cells per tile
constexpr int kCols = 9 * kNC;  // MMA columns (p, c), n = 8 p + c
constexpr int kWG = 4;          // tile pipelines (warpgroups) per CTA
constexpr uint32_t kWgCols = 128;  // TMEM columns per warpgroup

template <int ORD>
struct NbtDims {
  static constexpr int B = ORD * (ORD + 1) * (ORD + 2) / 6;
  static constexpr int Bp = (B + 3) / 4 * 4;
  static constexpr int F = ORD * (ORD + 1) / 2;
  static constexpr int FP = (F + 3) / 4 * 4;    // stored trace row
  static constexpr int KF = (FP + 7) / 8 * 8;   // K extent of one face
  static constexpr int K = 4 * KF;              // MMA K
  static constexpr int KC = K / 8;              // core-matrix chunks along K
  static constexpr int G = KF / 4;              // m per mixing thread: 4 groups per face, 128 threads
  static constexpr int V = G % 4 == 0 ? 4 : 2;  // floats per vector load of a trace row
  static constexpr int CS = 4 * 9 * FP + 4;     // cell stride of the trace tile (floats; +4 spreads banks)
  static constexpr size_t kOpA = (size_t)64 * K * 2 * 2;
  static constexpr size_t kX = (size_t)kNC * CS * 4;
  static constexpr size_t kBS = (size_t)kCols * K * 2 * 2;
  static constexpr size_t kWgBuf = ((kX > kBS ? kX : kBS) + 1023) / 1024 * 1024;  // trace tile, then B operand
  static constexpr size_t kAT = (size_t)kNC * 4 * 81 * 4;  // the tile's AminusT (or AplusT) rows
  static constexpr size_t kSmem = kOpA + kWG * (kWgBuf + 2 * kAT);
  static_assert(B <= 64, "M = 64 holds the basis");
  static_assert(K % 16 == 0 && G % 2 == 0 && G % V == 0, "whole MMA K steps, whole half2 pairs and vectors");
  static_assert(kX % 16 == 0 && kOpA % 1024 == 0 && kAT % 16 == 0, "16-byte regions");
};

template <int ORD, int FP, int F>
__device__ __forceinline__ void traceMap(int h, const float (&t)[FP], float (&s)[F]) {
  if constexpr (ORD == 4) sei_tcnb_o4::applyFp(h, t, s);
  if constexpr (ORD == 5) sei_tcnb_o5::applyFp(h, t, s);
  if constexpr (ORD == 6) sei_tcnb_o6::applyFp(h, t, s);
}

// Barrier of warpgroup wg (named barrier 1 + wg, 128 threads), optionally AND-reducing a flag.
__device__ __forceinline__ void wgSync(int wg) { asm volatile("bar.sync %0, 128;\n" ::"r"(1 + wg) : "memory"); }
__device__ __forceinline__ bool wgSyncAnd(int wg, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + wg)
      : "memory");
  return r != 0;
}

struct TileMeta {
  int reg[32];     // pair (c, i) = 4 c + i has a regular face with a neighbour trace
  int h[32];       // its orientation
  int sorted[32];  // regular pairs ordered by orientation
  int nsorted;
};

// One warp: metadata of tile `tile`, the bulk copies of its neighbour traces, L2 prefetch of its DOFs.
template <int ORD>
__device__ __forceinline__ void issueGather(const sei::TcNbArgs& A, int tile, float* X, TileMeta& meta, uint64_t* mbar) {
  using D = NbtDims<ORD>;
  const int lane = threadIdx.x & 31;
  const int c = lane >> 2, i = lane & 3;
  const int cell0 = tile * kNC;
  const int cnt = A.n - cell0 < kNC ? A.n - cell0 : kNC;
  const int cell = cell0 + c;
  int nb = -1, ft = 2, rl = 0;
  if (c < cnt) {
    const size_t f = (size_t)cell * 4 + i;
    nb = __ldg(A.nbr + f);
    ft = A.ftype[f];
    rl = A.rel[f];
  }
  const bool reg = c < cnt && ft == 0 && nb >= 0 && nb < A.ntotal;
  int h = rl >> 2;
  h = h > 2 ? 2 : h;
  const int j = rl & 3;
  meta.reg[lane] = reg ? 1 : 0;
  meta.h[lane] = h;
  // order the regular pairs by orientation (bucket offsets by ballot counts)
  const unsigned full = 0xffffffffu;
  const unsigned m0 = __ballot_sync(full, reg && h == 0), m1 = __ballot_sync(full, reg && h == 1),
                 m2 = __ballot_sync(full, reg && h == 2);
  const unsigned lt = (1u << lane) - 1u;
  const unsigned mine = h == 0 ? m0 : (h == 1 ? m1 : m2);
  const int base = h == 0 ? 0 : (h == 1 ? __popc(m0) : __popc(m0) + __popc(m1));
  if (reg) meta.sorted[base + __popc(mine & lt)] = lane;
  if (lane == 0) meta.nsorted = __popc(m0) + __popc(m1) + __popc(m2);
  const uint32_t rowBytes = 9 * D::FP * 4;
  const uint32_t total = (uint32_t)__popc(m0 | m1 | m2) * rowBytes;
  __syncwarp();
  if (lane == 0) sei_tc::mbarExpectTx(mbar, total);  // arrival + the transaction bytes, before any copy
  __syncwarp();
  if (reg)
    sei_tc::bulkCopyG2S(X + c * D::CS + i * 9 * D::FP, A.trace + ((size_t)j * A.ntotal + nb) * 9 * D::FP, rowBytes, mbar);
  if (lane == 0) sei_tc::prefetchL2(A.Q + (size_t)cell0 * 9 * D::Bp, (uint32_t)(cnt * 9 * D::Bp * 4));
}

// One thread: the bulk copies of tile `tile`'s flux matrices, AminusT (and AplusT with the local
// flux) of its cells, [cell][face][81] each, into the warpgroup's staging region.
template <int ORD>
__device__ __forceinline__ void issueFlux(const sei::TcNbArgs& A, int tile, float* Am, uint64_t* mbar) {
  using D = NbtDims<ORD>;
  const int cell0 = tile * kNC;
  const int cnt = A.n - cell0 < kNC ? A.n - cell0 : kNC;
  const uint32_t bytes = (uint32_t)cnt * 4 * 81 * 4;
  sei_tc::mbarExpectTx(mbar, A.aplus ? 2 * bytes : bytes);
  sei_tc::bulkCopyG2S(Am, A.aminus + (size_t)cell0 * 4 * 81, bytes, mbar);
  if (A.aplus) sei_tc::bulkCopyG2S(Am + D::kAT / 4, A.aplus + (size_t)cell0 * 4 * 81, bytes, mbar);
}

template <int ORD>
__global__ void __launch_bounds__(128 * kWG, 1) sei_nbt(sei::TcNbArgs A, const uint16_t* __restrict__ opA,
                                                        const float* __restrict__ scA) {
  using D = NbtDims<ORD>;
  constexpr int B = D::B, Bp = D::Bp, F = D::F, FP = D::FP, KC = D::KC, CS = D::CS;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbarTab, mbarLdAll[kWG], mbarMmaAll[kWG], mbarAAll[kWG];
  __shared__ uint32_t tslot;
  __shared__ TileMeta metaAll[kWG];
  __shared__ unsigned smaxAll[kWG][kCols];
  __shared__ float cscAll[kWG][kCols];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid >> 7, wt = tid & 127, ww = warp & 3;  // warpgroup, thread and warp in it
  uint16_t* aHi = reinterpret_cast<uint16_t*>(sm);
  uint16_t* aLo = aHi + 64 * D::K;
  unsigned char* buf = sm + D::kOpA + (size_t)wg * D::kWgBuf;
  float* X = reinterpret_cast<float*>(buf);
  uint16_t* bHi = reinterpret_cast<uint16_t*>(buf);  // the B operand replaces the trace tile
  uint16_t* bLo = bHi + kCols * D::K;
  uint64_t* mbarLd = &mbarLdAll[wg];
  uint64_t* mbarMma = &mbarMmaAll[wg];
  uint64_t* mbarA = &mbarAAll[wg];
  float* Am = reinterpret_cast<float*>(sm + D::kOpA + kWG * D::kWgBuf + (size_t)wg * 2 * D::kAT);  // AminusT, AplusT
  TileMeta& meta = metaAll[wg];
  unsigned* smax = smaxAll[wg];
  float* csc = cscAll[wg];
  if (warp == 0) sei_tc::tmemAlloc(&tslot, kWgCols * kWG);
  if (tid == 0) {
    sei_tc::mbarInit(&mbarTab, 1);
    for (int g = 0; g < kWG; ++g) {
      sei_tc::mbarInit(&mbarLdAll[g], 1);
      sei_tc::mbarInit(&mbarMmaAll[g], 1);
      sei_tc::mbarInit(&mbarAAll[g], 1);
    }
    sei_tc::mbarExpectTx(&mbarTab, (uint32_t)D::kOpA);
    sei_tc::bulkCopyG2S(aHi, opA, (uint32_t)D::kOpA, &mbarTab);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot + kWgCols * wg;
  // every wait's outcome is made uniform over the warpgroup, so its threads take the same path
  // through its barriers and the warp-collective TMEM loads
  bool ok = wgSyncAnd(wg, sei_tc::mbarWait(&mbarTab, 0, kMaxPolls));
  const bool tabPending = !ok;
  uint32_t ldPhase = 0, mmaPhase = 0, aPhase = 0;
  bool ldPending = false, mmaPending = false, aPending = false;
  const int ntiles = (A.n + kNC - 1) / kNC;
  const int stride = (int)gridDim.x * kWG;
  int tile = (int)blockIdx.x * kWG + wg;
  if (ok && tile < ntiles) {
    if (ww == 0) issueGather<ORD>(A, tile, X, meta, mbarLd);
    if (wt == 32) issueFlux<ORD>(A, tile, Am, mbarA);
    ldPending = aPending = true;
  }
  // epilogue row and column parity of this thread (M = 64: row 16 w + r on lane 32 w + r, r < 16;
  // the .16x64b load gives thread t row r = (t >> 2) + 8 (t & 1) and the columns of parity (t >> 1) & 1)
  const int kq = 16 * ww + (lane >> 2) + 8 * (lane & 1);
  const int es = (lane >> 1) & 1;
  const bool erow = kq < B;
  const float fsc = erow ? __ldg(scA + kq) : 0.f;
  for (; ok && tile < ntiles; tile += stride) {
    ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarLd, ldPhase, kMaxPolls));  // also: metadata visible
    if (!ok) break;
    ldPhase ^= 1;
    ldPending = false;
    const int cell0 = tile * kNC;
    const int cnt = A.n - cell0 < kNC ? A.n - cell0 : kNC;
    // ---- map: trace rows through fP_h diag(fM)^-1, in place
    if (wt < kCols) smax[wt] = 0u;
    const int nrows = meta.nsorted * 9;
    for (int it = wt; it < nrows; it += 128) {
      const int pr = meta.sorted[it / 9], q = it % 9;
      float* row = X + (pr >> 2) * CS + ((pr & 3) * 9 + q) * FP;
      float t[FP];
#pragma unroll
      for (int u = 0; u < FP / 4; ++u) {
        const float4 v = reinterpret_cast<const float4*>(row)[u];
        t[4 * u] = v.x;
        t[4 * u + 1] = v.y;
        t[4 * u + 2] = v.z;
        t[4 * u + 3] = v.w;
      }
      float s[F];
      traceMap<ORD>(meta.h[pr], t, s);
#pragma unroll
      for (int u = 0; u < FP / 4; ++u)
        reinterpret_cast<float4*>(row)[u] =
            make_float4(4 * u < F ? s[4 * u < F ? 4 * u : 0] : 0.f, 4 * u + 1 < F ? s[4 * u + 1 < F ? 4 * u + 1 : 0] : 0.f,
                        4 * u + 2 < F ? s[4 * u + 2 < F ? 4 * u + 2 : 0] : 0.f,
                        4 * u + 3 < F ? s[4 * u + 3 < F ? 4 * u + 3 : 0] : 0.f);
    }
    wgSync(wg);
    // ---- mix: S[m, (p, c)] for the G = KF / 4 m of this thread's group: thread (cell c, face
    // fi = warp, group mg = lane / 8), all 128 threads of the warpgroup busy
    ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarA, aPhase, kMaxPolls));
    if (!ok) break;
    aPhase ^= 1;
    aPending = false;
    constexpr int G = D::G, V = D::V;
    const int c = wt & 7, fi = ww, mg = lane >> 3;
    float S[G][9];
#pragma unroll
    for (int u = 0; u < G; ++u)
#pragma unroll
      for (int p = 0; p < 9; ++p) S[u][p] = 0.f;
    if (A.aplus && c < cnt) {
      // local flux of face fi from the cell's own trace: S += T_fi AplusT_fi (zero on DR faces)
      const float* tr = A.trace + (((size_t)fi * A.ntotal + A.first + cell0 + c) * 9) * FP + G * mg;
      const float* ap = Am + D::kAT / 4 + (c * 4 + fi) * 81;
#pragma unroll 3
      for (int q = 0; q < 9; ++q) {
        float r[G];
#pragma unroll
        for (int h = 0; h < G / V; ++h) {
          if (G * mg + V * h < FP) {  // whole chunks inside the stored row
            if constexpr (V == 4) {
              const float4 y = __ldg(reinterpret_cast<const float4*>(tr + q * FP + 4 * h));
              r[4 * h] = y.x;
              r[4 * h + 1] = y.y;
              r[4 * h + 2] = y.z;
              r[4 * h + 3] = y.w;
            } else {
              const float2 y = __ldg(reinterpret_cast<const float2*>(tr + q * FP + 2 * h));
              r[2 * h] = y.x;
              r[2 * h + 1] = y.y;
            }
          } else {
#pragma unroll
            for (int e = 0; e < V; ++e) r[V * h + e] = 0.f;
          }
        }
#pragma unroll
        for (int p = 0; p < 9; ++p) {
          const float a = ap[q + 9 * p];
#pragma unroll
          for (int u = 0; u < G; ++u) S[u][p] = fmaf(r[u], a, S[u][p]);
        }
      }
    }
    if (meta.reg[4 * c + fi]) {
      const float* xr = X + c * CS + fi * 9 * FP + G * mg;
      const float* am = Am + (c * 4 + fi) * 81;
#pragma unroll 3
      for (int q = 0; q < 9; ++q) {
        float r[G];
#pragma unroll
        for (int h = 0; h < G / V; ++h) {
          if constexpr (V == 4) {
            const float4 y = reinterpret_cast<const float4*>(xr + q * FP)[h];
            r[4 * h] = y.x;
            r[4 * h + 1] = y.y;
            r[4 * h + 2] = y.z;
            r[4 * h + 3] = y.w;
          } else {
            const float2 y = reinterpret_cast<const float2*>(xr + q * FP)[h];
            r[2 * h] = y.x;
            r[2 * h + 1] = y.y;
          }
        }
#pragma unroll
        for (int u = 0; u < G; ++u)
          if (G * mg + u >= F) r[u] = 0.f;  // past the face basis (the next row at orders 4 and 5)
#pragma unroll
        for (int p = 0; p < 9; ++p) {
          const float a = am[q + 9 * p];
#pragma unroll
          for (int u = 0; u < G; ++u) S[u][p] = fmaf(r[u], a, S[u][p]);
        }
      }
    }
    // column maxima over this warp's groups of cell c, then over the warps (faces)
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      float mx = 0.f;
#pragma unroll
      for (int u = 0; u < G; ++u) mx = fmaxf(mx, fabsf(S[u][p]));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
      if (lane < 8) atomicMax(&smax[8 * p + c], __float_as_uint(mx));
    }
    wgSync(wg);  // the maxima are complete and every read of the trace tile and flux matrices is done
    // the flux matrices of the warpgroup's next tile overlap the split, MMA and epilogue
    if (tile + stride < ntiles) {
      if (wt == 32) issueFlux<ORD>(A, tile + stride, Am, mbarA);
      aPending = true;
    }
    if (wt < kCols) csc[wt] = sei_tc::pow2(sei_tc::pow2Exp(__uint_as_float(smax[wt])));
    {
      // K index fi KF + G mg + u; the core matrix of 8 k holds k % 8 at 2-byte steps, so each
      // pair (u, u + 1) is one aligned 4-byte store
#pragma unroll
      for (int p = 0; p < 9; ++p) {
        const float sc = sei_tc::pow2(-sei_tc::pow2Exp(__uint_as_float(smax[8 * p + c])));
#pragma unroll
        for (int u = 0; u < G; u += 2) {
          const float x0 = S[u][p] * sc, x1 = S[u + 1][p] * sc;
          const __half2 h2 = __floats2half2_rn(x0, x1);
          const float2 b2 = __half22float2(h2);
          const __half2 l2 = __floats2half2_rn(x0 - b2.x, x1 - b2.y);
          const int kk = fi * D::KF + G * mg + u;
          const uint32_t off = ((uint32_t)(p * KC + kk / 8) * 128 + (uint32_t)c * 16) / 2 + (uint32_t)(kk % 8);
          *reinterpret_cast<__half2*>(bHi + off) = h2;
          *reinterpret_cast<__half2*>(bLo + off) = l2;
        }
      }
    }
    sei_tc::fenceProxyAsync();
    sei_tc::fenceBeforeSync();
    wgSync(wg);
    sei_tc::fenceAfterSync();
    if (wt == 0) {
      constexpr uint32_t idesc = sei_tc::idescF16(64, kCols);
      const uint32_t sbo = (uint32_t)KC * 128;
      const uint32_t pa[3] = {sei_tc::smemAddr(aHi), sei_tc::smemAddr(aHi), sei_tc::smemAddr(aLo)};
      const uint32_t pb[3] = {sei_tc::smemAddr(bHi), sei_tc::smemAddr(bLo), sei_tc::smemAddr(bHi)};
#pragma unroll 1
      for (int s = 0; s < D::K / 16; ++s)
#pragma unroll
        for (int t = 0; t < 3; ++t)
          sei_tc::mmaSSf16(taddr, sei_tc::smemDesc(pa[t] + 256 * s, 128, sbo), sei_tc::smemDesc(pb[t] + 256 * s, 128, sbo),
                           idesc, s > 0 || t > 0);
      sei_tc::mmaCommit(mbarMma);
    }
    mmaPending = true;
    // ---- epilogue: row k adds D[k, (p, c)] to Q[c][p][k] by reductions in L2 (the tile's DOFs
    // were prefetched there by the gather); register j holds column n = 2 j + es, i.e. p = j / 4
    // and c = 2 (j % 4) + es
    float* Qr = A.Q + ((size_t)cell0 * 9 + (size_t)es * 9) * Bp + kq;
    ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarMma, mmaPhase, kMaxPolls));
    if (!ok) break;
    mmaPhase ^= 1;
    mmaPending = false;
    sei_tc::fenceAfterSync();
    // the B operand is consumed: the next tile's gather overlaps this epilogue
    const int next = tile + stride;
    if (next < ntiles) {
      if (ww == 0) issueGather<ORD>(A, next, X, meta, mbarLd);
      ldPending = true;
    }
    {
      const uint32_t tb = taddr + ((uint32_t)(32 * ww) << 16);
      float v[36];
      sei_tc::tmemLoad16x64b32(tb, v);
      sei_tc::tmemLoad16x64b4(tb + 64u, v + 32);
      sei_tc::tmemLoadWait();
#pragma unroll
      for (int j = 0; j < 36; ++j) {
        const int cc = 2 * (j & 3) + es;
        if (erow && cc < cnt) atomicAdd(Qr + (size_t)(18 * (j & 3) + (j >> 2)) * Bp, v[j] * fsc * csc[2 * j + es]);
      }
    }
    sei_tc::fenceBeforeSync();
    wgSync(wg);
    sei_tc::fenceAfterSync();
  }
  if (!ok) {
    if (wt == 0) atomicExch(A.status, 1);
    // copies or MMAs issued before the wait that gave up may still be in flight: give them a
    // second bounded wait before the tensor memory is freed and the shared memory released
    if (tabPending) (void)sei_tc::mbarWait(&mbarTab, 0, kMaxPolls);
    if (ldPending) (void)sei_tc::mbarWait(mbarLd, ldPhase, kMaxPolls);
    if (aPending) (void)sei_tc::mbarWait(mbarA, aPhase, kMaxPolls);
    if (mmaPending) (void)sei_tc::mbarWait(mbarMma, mmaPhase, kMaxPolls);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (warp == 0) sei_tc::tmemDealloc(tslot, kWgCols * kWG);
}

template <int ORD>
int launchNbt(const sei::DeviceArrays& d, const float* trace, int* status, int sms, void* stream, const void* opSym,
              const void* scSym, bool withLocalFlux) {
  using Dm = NbtDims<ORD>;
  sei::TcNbArgs a{};
  a.n = d.n;
  a.ntotal = d.ntotal > 0 ? d.ntotal : d.n;
  a.first = d.first;
  a.aplus = withLocalFlux ? d.aplus : nullptr;
  a.Q = d.Q;
  a.trace = trace;
  a.aminus = d.aminus;
  a.nbr = d.nbr;
  a.rel = d.rel;
  a.ftype = d.ftype;
  a.status = status;
  void* op = nullptr;
  void* sc = nullptr;
  if (cudaGetSymbolAddress(&op, opSym) != cudaSuccess || cudaGetSymbolAddress(&sc, scSym) != cudaSuccess) return -1;
  if (cudaFuncSetAttribute(sei_nbt<ORD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Dm::kSmem) != cudaSuccess)
    return -1;
  const int ntiles = (d.n + kNC - 1) / kNC;
  const int need = (ntiles + kWG - 1) / kWG;
  const int grid = need < sms ? need : sms;
  if (grid <= 0) return 0;
  sei_nbt<ORD><<<grid, 128 * kWG, Dm::kSmem, (cudaStream_t)stream>>>(a, (const uint16_t*)op, (const float*)sc);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

namespace sei {

int launchNeighborTransposed(int order, const DeviceArrays& d, const float* trace, int* status, int sms, void* stream,
                             bool withLocalFlux) {
  switch (order) {
    case 4:
      return launchNbt<4>(d, trace, status, sms, stream, (const void*)&sei_tc_o4::knbt_op, (const void*)&sei_tc_o4::knbt_scale,
                          withLocalFlux);
    case 5:
      return launchNbt<5>(d, trace, status, sms, stream, (const void*)&sei_tc_o5::knbt_op, (const void*)&sei_tc_o5::knbt_scale,
                          withLocalFlux);
    case 6:
      return launchNbt<6>(d, trace, status, sms, stream, (const void*)&sei_tc_o6::knbt_op, (const void*)&sei_tc_o6::knbt_scale,
                          withLocalFlux);
    default:
      return -1;
  }
}

}  // namespace sei
