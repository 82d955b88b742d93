// Volume integral and local flux on the tensor cores in the transposed form
// (Local::computeIntegral, codegen/kernels/aderdg.py:337-386), which also writes the face traces
// T_f = fMrT_f I of every cell for the neighbour kernel of the mixed-precision path.
//
// A tile is 3 cells.  Every MMA puts a basis index on the TMEM lanes and the tile's
// (cell c, quantity q) pairs on 32 columns (n = 9 c + q; columns 27..31 unused):
//   Z_d[k, n] = sum_l kDivM_d[k, l] I[l, n]        d = 0, 1, 2   (M = 64, K = 64)
//   T[(f, m), n] = sum_l rT_f[m, l] I[l, n]          traces      (M = 128, K = 64)
//   L[k, n] = sum_{f, m} rT_f[m, k] S_f[m, n]        lift        (M = 64, K = 4 KF; the rT table
//                                                     read MN-major, rDivM_f = diag(1/M) rT_f^T)
// with, on the CUDA cores in FP32,
//   vol[k, (c, p)] = sum_d sum_q Z_d[k, (c, q)] star_d[c][q, p]      (lane k, registers)
//   S_f[m, (c, p)] = sum_q fM_m T[(f, m), (c, q)] AplusT_f[c][q, p]   (thread (c, f, octet of m))
// and Q += vol + diag(1/M) L.  The products are split FP16 x3 (hi hi + hi lo + lo hi, FP32
// accumulation in TMEM); the tables arrive pre-split with one power-of-two scale per row, the
// data get one per column (the maximum of the column over K).
//
// A CTA (one per SM) stages the tables once and runs four independent tile pipelines, one per
// warpgroup, each with its own B-operand buffer, star tile, 128 TMEM columns, mbarriers and
// named barrier, so the pipelines overlap one another's copy and MMA waits.  Per tile:
//   produce  one warp, thread (c, octet of l): I from global -> FP16 hi/lo B operand (K-major);
//   MMA 1    one thread: the three Z_d and T (TMEM columns 0..95 and 96..127 of the warpgroup);
//   epilogue lane (f, m): the traces to global ([face][cell][9][FP]); lane k: vol, parked in the
//            columns of Z_0;
//   mix      thread (c, f, octet of m): re-reads its cell's traces (L2) and AplusT, S_f into the
//            lift's B operand (over the first B operand);
//   MMA 2    the lift into columns 96..127;
//   epilogue lane k: Q[c][p][k] += vol + L / M_k.
//
// Failure handling: every mbarrier wait is bounded and its outcome made uniform over the
// warpgroup (barrier reduction); a wait that gives up sets the status word, waits once more
// (bounded) for the copies and MMAs in flight and leaves the tile loop; the tensor memory is freed
// after all warpgroups have left.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"
#include "_gen/tc_tables_o4.cuh"
#include "_gen/tc_tables_o5.cuh"
#include "_gen/tc_tables_o6.cuh"

namespace {

constexpr uint32_t kMaxPolls = 1u << 26;
constexpr int kNC = 3;   // cells per tile
constexpr int kN = 32;   // MMA columns, n = 9 c + q
constexpr int kUsed = 9 * kNC;
constexpr int kWG = 4;   // tile pipelines (warpgroups) per CTA
constexpr uint32_t kWgCols = 128;
constexpr int kColT = 96;  // TMEM column (within the warpgroup's) of the traces and of the lift

// Non-zeros of the elastic star matrix in their stored order: source quantity q, target p
// (codegen/matrices/star.xml; the same order as sei::kStarNz).
__host__ __device__ constexpr int kStarQ(int j) {
  constexpr int t[24] = {6, 7, 8, 6, 7, 8, 6, 7, 8, 6, 7, 7, 8, 6, 8, 0, 3, 5, 1, 3, 4, 2, 4, 5};
  return t[j];
}
__host__ __device__ constexpr int kStarP(int j) {
  constexpr int t[24] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 6, 7, 7, 7, 8, 8, 8};
  return t[j];
}

struct LtArgs {
  int n;
  float* Q;
  const float* I;
  const float* star_nz;
  const float* aplus;
  float* trace;  // [4][tplane][9][FP] (points at this launch's first cell)
  int tplane;
  int traceOnly;
  int* status;
  const uint16_t* opVol;  // kDivM_d blocks, hi then lo
  const float* scVol;     // [192] row scales
  const uint16_t* opRt;   // rT stack, hi then lo
  const float* scRt;      // [128] row scales
  const float* tsc;       // [128] row scale x fM_m
  const float* invm;      // [64] 1 / M_k
};

template <int ORD>
struct LtDims {
  static constexpr int B = ORD * (ORD + 1) * (ORD + 2) / 6;
  static constexpr int Bp = (B + 3) / 4 * 4;
  static constexpr int F = ORD * (ORD + 1) / 2;
  static constexpr int FP = (F + 3) / 4 * 4;
  static constexpr int KF = (FP + 7) / 8 * 8;
  static constexpr int KT = 4 * KF;  // lift K
  static constexpr int KTC = KT / 8;
  static constexpr int OCT = KF / 8;
  static constexpr int ITEMS = 4 * 4 * OCT;  // mixing threads, c = 0..3 (c = 3 writes unused columns)
  static constexpr size_t kVolA = (size_t)192 * 64 * 2 * 2;
  static constexpr size_t kRtA = (size_t)128 * 64 * 2 * 2;
  static constexpr size_t kBI = (size_t)kN * 64 * 2 * 2;
  static constexpr size_t kBS = (size_t)kN * KT * 2 * 2;
  static constexpr size_t kB = kBI > kBS ? kBI : kBS;
  static constexpr size_t kStar = 1024;  // 3 cells x 72 floats
  static constexpr size_t kWgBuf = kB + kStar;
  static constexpr size_t kSmem = kVolA + kRtA + kWG * kWgBuf;
  static_assert(B <= 64 && 4 * KF <= 128 && KT % 16 == 0 && ITEMS <= 64, "tile shapes");
  static_assert(kB % 1024 == 0, "aligned per-warpgroup buffers");
};

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

__device__ __forceinline__ int expOf(float m) { return sei_tc::pow2Exp(m); }

// Splits 8 values (times 2^-e) into FP16 hi and lo and stores them as one 16-byte row chunk each.
__device__ __forceinline__ void storeSplit8(uint16_t* hiBase, uint16_t* loBase, uint32_t offBytes, const float (&x)[8],
                                            int e) {
  uint32_t hw[4], lw[4];
  const float sc = sei_tc::pow2(-e);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float x0 = x[2 * u] * sc, x1 = x[2 * u + 1] * sc;
    const __half2 h2 = __floats2half2_rn(x0, x1);
    const float2 b2 = __half22float2(h2);
    const __half2 l2 = __floats2half2_rn(x0 - b2.x, x1 - b2.y);
    hw[u] = *reinterpret_cast<const uint32_t*>(&h2);
    lw[u] = *reinterpret_cast<const uint32_t*>(&l2);
  }
  *reinterpret_cast<uint4*>(hiBase + offBytes / 2) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  *reinterpret_cast<uint4*>(loBase + offBytes / 2) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// 32 consecutive TMEM columns of this thread's lane (load, store).
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float (&v)[32]) {
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float w[16];
    sei_tc::tmemLoad16(taddr + 16 * j, w);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[16 * j + i] = w[i];
  }
  sei_tc::tmemLoadWait();
}
__device__ __forceinline__ void tmemStore32(uint32_t taddr, const float (&v)[32]) {
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float w[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] = v[16 * j + i];
    sei_tc::tmemStore16(taddr + 16 * j, w);
  }
  sei_tc::tmemStoreWait();
}

// One thread: the tile's star non-zeros into shared memory, L2 prefetch of its I and Q.
template <int ORD>
__device__ __forceinline__ void issueTileLoad(const LtArgs& A, int tile, float* starT, uint64_t* mbar) {
  using D = LtDims<ORD>;
  const int cell0 = tile * kNC;
  const int cnt = A.n - cell0 < kNC ? A.n - cell0 : kNC;
  const uint32_t bytes = (uint32_t)cnt * 72 * 4;
  sei_tc::mbarExpectTx(mbar, bytes);
  sei_tc::bulkCopyG2S(starT, A.star_nz + (size_t)cell0 * 72, bytes, mbar);
  sei_tc::prefetchL2(A.I + (size_t)cell0 * 9 * D::Bp, (uint32_t)(cnt * 9 * D::Bp * 4));
  sei_tc::prefetchL2(A.Q + (size_t)cell0 * 9 * D::Bp, (uint32_t)(cnt * 9 * D::Bp * 4));
}

template <int ORD>
__global__ void __launch_bounds__(128 * kWG, 1) sei_lintt(LtArgs A) {
  using D = LtDims<ORD>;
  constexpr int B = D::B, Bp = D::Bp, F = D::F, FP = D::FP, KF = D::KF, OCT = D::OCT, KTC = D::KTC;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbarTab, mbarLdAll[kWG], mbarMmaAll[kWG];
  __shared__ uint32_t tslot;
  __shared__ unsigned smaxAll[kWG][kN];
  __shared__ float escIAll[kWG][kN], escSAll[kWG][kN];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = tid >> 7, wt = tid & 127, ww = warp & 3;  // warpgroup, thread and warp in it
  uint16_t* volHi = reinterpret_cast<uint16_t*>(sm);
  uint16_t* volLo = volHi + 192 * 64;
  uint16_t* rtHi = reinterpret_cast<uint16_t*>(sm + D::kVolA);
  uint16_t* rtLo = rtHi + 128 * 64;
  unsigned char* buf = sm + D::kVolA + D::kRtA + (size_t)wg * D::kWgBuf;
  uint16_t* bHi = reinterpret_cast<uint16_t*>(buf);
  uint16_t* biLo = bHi + kN * 64;       // lo half of the first B operand (I)
  uint16_t* bsLo = bHi + kN * D::KT;    // lo half of the lift's B operand (S)
  float* starT = reinterpret_cast<float*>(buf + D::kB);
  uint64_t* mbarLd = &mbarLdAll[wg];
  uint64_t* mbarMma = &mbarMmaAll[wg];
  unsigned* smax = smaxAll[wg];
  float* escI = escIAll[wg];
  float* escS = escSAll[wg];
  if (warp == 0) sei_tc::tmemAlloc(&tslot, kWgCols * kWG);
  if (tid == 0) {
    sei_tc::mbarInit(&mbarTab, 1);
    for (int g = 0; g < kWG; ++g) {
      sei_tc::mbarInit(&mbarLdAll[g], 1);
      sei_tc::mbarInit(&mbarMmaAll[g], 1);
    }
    sei_tc::mbarExpectTx(&mbarTab, (uint32_t)(D::kVolA + D::kRtA));
    sei_tc::bulkCopyG2S(volHi, A.opVol, (uint32_t)D::kVolA, &mbarTab);
    sei_tc::bulkCopyG2S(rtHi, A.opRt, (uint32_t)D::kRtA, &mbarTab);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  sei_tc::fenceAfterSync();
  const uint32_t taddr = tslot + kWgCols * wg;
  const uint32_t tlane = taddr + ((uint32_t)(32 * ww) << 16);
  bool ok = wgSyncAnd(wg, sei_tc::mbarWait(&mbarTab, 0, kMaxPolls));
  const bool tabPending = !ok;
  uint32_t ldPhase = 0, mmaPhase = 0;
  bool ldPending = false, mmaPending = false;
  const int ntiles = (A.n + kNC - 1) / kNC;
  const int stride = (int)gridDim.x * kWG;
  int tile = (int)blockIdx.x * kWG + wg;
  if (ok && tile < ntiles) {
    if (wt == 0) issueTileLoad<ORD>(A, tile, starT, mbarLd);
    ldPending = true;
  }
  // lane roles: k = 16 w + t (t < 16) for the M = 64 results; r = 32 w + t for the traces
  const int kq = lane < 16 ? 16 * ww + lane : -1;
  const bool vrow = kq >= 0 && kq < B;
  float fd0 = 0.f, fd1 = 0.f, fd2 = 0.f, invM = 0.f;
  if (vrow) {
    fd0 = __ldg(A.scVol + kq);
    fd1 = __ldg(A.scVol + 64 + kq);
    fd2 = __ldg(A.scVol + 128 + kq);
    invM = __ldg(A.invm + kq);
  }
  const int r = wt, ti = r / KF, tm = r % KF;
  const bool trow = r < 4 * KF && tm < FP;
  const float tscale = r < 4 * KF ? __ldg(A.tsc + r) : 0.f;
  for (; ok && tile < ntiles; tile += stride) {
    ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarLd, ldPhase, kMaxPolls));
    if (!ok) break;
    ldPhase ^= 1;
    ldPending = false;
    const int cell0 = tile * kNC;
    const int cnt = A.n - cell0 < kNC ? A.n - cell0 : kNC;
    if (wt < kN) smax[wt] = 0u;
    // ---- produce (warp 0): I -> B operand rows n = 9 c + q, K chunk = octet of l; the row
    // maxima over the 8 octets are warp shuffles (lane = c + 4 octet)
    if (ww == 0) {
      const int pc = lane & 3, po = lane >> 2;
      // all 18 loads of this thread in flight at once
      float vv[9][8];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
#pragma unroll
        for (int u = 0; u < 8; ++u) vv[q][u] = 0.f;
        if (pc < cnt) {
          const float* row = A.I + ((size_t)(cell0 + pc) * 9 + q) * Bp + 8 * po;
#pragma unroll
          for (int h = 0; h < 2; ++h)
            if (8 * po + 4 * h < Bp) {
              const float4 x = __ldg(reinterpret_cast<const float4*>(row) + h);
              vv[q][4 * h] = x.x;
              vv[q][4 * h + 1] = x.y;
              vv[q][4 * h + 2] = x.z;
              vv[q][4 * h + 3] = x.w;
            }
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (8 * po + u >= B) vv[q][u] = 0.f;
        }
      }
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = vv[q][u];
        float mx = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) mx = fmaxf(mx, fabsf(v[u]));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 4));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
        const int e = expOf(mx);
        if (pc < kNC) {
          const int n = 9 * pc + q;
          storeSplit8(bHi, biLo, (uint32_t)(((n >> 3) * 8 + po) * 128 + (n & 7) * 16), v, e);
          if (po == 0) escI[n] = sei_tc::pow2(e);
        } else if (q < kN - kUsed) {
          const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          const int n = kUsed + q;  // unused columns 27..31
          storeSplit8(bHi, biLo, (uint32_t)(((n >> 3) * 8 + po) * 128 + (n & 7) * 16), z, 0);
        }
      }
    }
    sei_tc::fenceProxyAsync();
    sei_tc::fenceBeforeSync();
    wgSync(wg);
    sei_tc::fenceAfterSync();
    // ---- MMA 1: Z_0, Z_1, Z_2 (M = 64) and the traces (M = 128)
    if (wt == 0) {
      const uint32_t sbo = 8 * 128;
      const uint32_t pb[3] = {sei_tc::smemAddr(bHi), sei_tc::smemAddr(biLo), sei_tc::smemAddr(bHi)};
      if (!A.traceOnly) {
        constexpr uint32_t id64 = sei_tc::idescF16(64, kN);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const uint32_t pa[3] = {sei_tc::smemAddr(volHi) + 8192u * d, sei_tc::smemAddr(volHi) + 8192u * d,
                                  sei_tc::smemAddr(volLo) + 8192u * d};
#pragma unroll
          for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int t = 0; t < 3; ++t)
              sei_tc::mmaSSf16(taddr + 32 * d, sei_tc::smemDesc(pa[t] + 256 * s, 128, sbo),
                               sei_tc::smemDesc(pb[t] + 256 * s, 128, sbo), id64, s > 0 || t > 0);
        }
      }
      constexpr uint32_t id128 = sei_tc::idescF16(128, kN);
      const uint32_t pa[3] = {sei_tc::smemAddr(rtHi), sei_tc::smemAddr(rtHi), sei_tc::smemAddr(rtLo)};
#pragma unroll
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int t = 0; t < 3; ++t)
          sei_tc::mmaSSf16(taddr + kColT, sei_tc::smemDesc(pa[t] + 256 * s, 128, sbo),
                           sei_tc::smemDesc(pb[t] + 256 * s, 128, sbo), id128, s > 0 || t > 0);
      sei_tc::mmaCommit(mbarMma);
    }
    mmaPending = true;
    ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarMma, mmaPhase, kMaxPolls));
    if (!ok) break;
    mmaPhase ^= 1;
    mmaPending = false;
    sei_tc::fenceAfterSync();
    // ---- epilogue 1: traces out (lane (f, m)); volume of lane k parked in the columns of Z_0
    {
      float t[32];
      tmemLoad32(tlane + kColT, t);
      if (trow) {
#pragma unroll
        for (int c = 0; c < kNC; ++c)
          if (c < cnt) {
            float* dst = A.trace + (((size_t)ti * A.tplane + cell0 + c) * 9) * FP + tm;
#pragma unroll
            for (int q = 0; q < 9; ++q) dst[q * FP] = t[9 * c + q] * tscale * escI[9 * c + q];
          }
      }
    }
    if (!A.traceOnly) {
      float vol[32];
#pragma unroll
      for (int n = 0; n < 32; ++n) vol[n] = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float z[32];
        tmemLoad32(tlane + 32 * d, z);
        const float fdd = d == 0 ? fd0 : (d == 1 ? fd1 : fd2);
#pragma unroll
        for (int n = 0; n < kUsed; ++n) z[n] *= fdd * escI[n];
#pragma unroll
        for (int c = 0; c < kNC; ++c) {
          const float4* st4 = reinterpret_cast<const float4*>(starT + c * 72 + 24 * d);
          float st[24];
#pragma unroll
          for (int j4 = 0; j4 < 6; ++j4) {
            const float4 s4 = st4[j4];
            st[4 * j4] = s4.x;
            st[4 * j4 + 1] = s4.y;
            st[4 * j4 + 2] = s4.z;
            st[4 * j4 + 3] = s4.w;
          }
#pragma unroll
          for (int j = 0; j < 24; ++j) vol[9 * c + kStarP(j)] = fmaf(st[j], z[9 * c + kStarQ(j)], vol[9 * c + kStarP(j)]);
        }
      }
      tmemStore32(tlane, vol);
    }
    sei_tc::fenceBeforeSync();
    wgSync(wg);  // traces written and visible to the warpgroup; TMEM and the star tile read
    sei_tc::fenceAfterSync();
    {
      const int next = tile + stride;
      if (next < ntiles) {
        if (wt == 0) issueTileLoad<ORD>(A, next, starT, mbarLd);
        ldPending = true;
      }
    }
    if (!A.traceOnly) {
      // ---- mix (two warps): S_f[m, (c, p)] for this thread's cell, face and octet of m
      const int c = wt & 3, g = wt >> 2, fi = g / OCT, oc = g % OCT;
      if (wt < 64) {
        float S[8][9];
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int p = 0; p < 9; ++p) S[u][p] = 0.f;
        if (wt < D::ITEMS && c < cnt) {
          const float* tr = A.trace + (((size_t)fi * A.tplane + cell0 + c) * 9) * FP + 8 * oc;
          const float* am = A.aplus + ((size_t)(cell0 + c) * 4 + fi) * 81;
#pragma unroll 3
          for (int q = 0; q < 9; ++q) {
            float x[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 2; ++h)
              if (8 * oc + 4 * h < FP) {
                const float4 y = __ldcg(reinterpret_cast<const float4*>(tr + q * FP) + h);
                x[4 * h] = y.x;
                x[4 * h + 1] = y.y;
                x[4 * h + 2] = y.z;
                x[4 * h + 3] = y.w;
              }
#pragma unroll
            for (int p = 0; p < 9; ++p) {
              const float a = __ldg(am + q + 9 * p);
#pragma unroll
              for (int u = 0; u < 8; ++u) S[u][p] = fmaf(x[u], a, S[u][p]);
            }
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float comp = 8 * oc + u < F ? __ldg(A.scRt + KF * fi + 8 * oc + u) : 0.f;
#pragma unroll
            for (int p = 0; p < 9; ++p) S[u][p] *= comp;
          }
        }
#pragma unroll
        for (int p = 0; p < 9; ++p) {
          float mx = 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) mx = fmaxf(mx, fabsf(S[u][p]));
          mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 4));
          mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
          mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
          if (lane < kNC) atomicMax(&smax[9 * c + p], __float_as_uint(mx));
        }
        wgSync(wg);  // the maxima are complete (the other warps wait at the barrier below)
        if (wt < D::ITEMS) {
          const int j = fi * OCT + oc;
          if (c < kNC) {
#pragma unroll
            for (int p = 0; p < 9; ++p) {
              const int n = 9 * c + p;
              const int e = expOf(__uint_as_float(smax[n]));
              float x[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) x[u] = S[u][p];
              storeSplit8(bHi, bsLo, (uint32_t)(((n >> 3) * KTC + j) * 128 + (n & 7) * 16), x, e);
              if (g == 0) escS[n] = sei_tc::pow2(e);
            }
          } else {
            const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int n = kUsed; n < kN; ++n)  // unused columns 27..31
              storeSplit8(bHi, bsLo, (uint32_t)(((n >> 3) * KTC + j) * 128 + (n & 7) * 16), z, 0);
          }
        }
      } else {
        wgSync(wg);
      }
      sei_tc::fenceProxyAsync();
      sei_tc::fenceBeforeSync();
      wgSync(wg);
      sei_tc::fenceAfterSync();
      // ---- MMA 2: the lift, rT table read MN-major (M = basis k, K = (f, m))
      if (wt == 0) {
        constexpr uint32_t idl = sei_tc::idescF16Major(64, kN, 1, 0);
        const uint32_t pa[3] = {sei_tc::smemAddr(rtHi), sei_tc::smemAddr(rtHi), sei_tc::smemAddr(rtLo)};
        const uint32_t pb[3] = {sei_tc::smemAddr(bHi), sei_tc::smemAddr(bsLo), sei_tc::smemAddr(bHi)};
        const uint32_t sboB = (uint32_t)KTC * 128;
#pragma unroll
        for (int s = 0; s < D::KT / 16; ++s)
#pragma unroll
          for (int t = 0; t < 3; ++t)
            sei_tc::mmaSSf16(taddr + kColT, sei_tc::smemDesc(pa[t] + 2048 * s, 1024, 128),
                             sei_tc::smemDesc(pb[t] + 256 * s, 128, sboB), idl, s > 0 || t > 0);
        sei_tc::mmaCommit(mbarMma);
      }
      mmaPending = true;
      // Q of the tile for the epilogue, loaded while the lift runs
      float qv[kUsed];
#pragma unroll
      for (int n = 0; n < kUsed; ++n)
        qv[n] = (vrow && n / 9 < cnt) ? A.Q[((size_t)(cell0 + n / 9) * 9 + n % 9) * Bp + kq] : 0.f;
      ok = wgSyncAnd(wg, sei_tc::mbarWait(mbarMma, mmaPhase, kMaxPolls));
      if (!ok) break;
      mmaPhase ^= 1;
      mmaPending = false;
      sei_tc::fenceAfterSync();
      // ---- epilogue 2: Q += vol + L / M_k
      float L[32], vol[32];
      tmemLoad32(tlane + kColT, L);
      tmemLoad32(tlane, vol);
      if (vrow) {
#pragma unroll
        for (int n = 0; n < kUsed; ++n)
          if (n / 9 < cnt) A.Q[((size_t)(cell0 + n / 9) * 9 + n % 9) * Bp + kq] = qv[n] + vol[n] + L[n] * escS[n] * invM;
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
    if (mmaPending) (void)sei_tc::mbarWait(mbarMma, mmaPhase, kMaxPolls);
  }
  sei_tc::fenceBeforeSync();
  __syncthreads();
  if (warp == 0) sei_tc::tmemDealloc(tslot, kWgCols * kWG);
}

template <int ORD>
int launchLintt(const sei::DeviceArrays& d, float* trace, int traceOnly, int* status, int sms, void* stream,
                const void* opVol, const void* scVol, const void* opRt, const void* scRt, const void* tsc,
                const void* invm) {
  using Dm = LtDims<ORD>;
  LtArgs a{};
  a.n = d.n;
  a.Q = d.Q;
  a.I = d.I;
  a.star_nz = d.star_nz;
  a.aplus = d.aplus;
  a.trace = trace;
  a.tplane = d.ntotal > 0 ? d.ntotal : d.n;
  a.traceOnly = traceOnly;
  a.status = status;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, opVol) != cudaSuccess) return -1;
  a.opVol = (const uint16_t*)p;
  if (cudaGetSymbolAddress(&p, scVol) != cudaSuccess) return -1;
  a.scVol = (const float*)p;
  if (cudaGetSymbolAddress(&p, opRt) != cudaSuccess) return -1;
  a.opRt = (const uint16_t*)p;
  if (cudaGetSymbolAddress(&p, scRt) != cudaSuccess) return -1;
  a.scRt = (const float*)p;
  if (cudaGetSymbolAddress(&p, tsc) != cudaSuccess) return -1;
  a.tsc = (const float*)p;
  if (cudaGetSymbolAddress(&p, invm) != cudaSuccess) return -1;
  a.invm = (const float*)p;
  if (!trace) return -1;
  if (cudaFuncSetAttribute(sei_lintt<ORD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Dm::kSmem) != cudaSuccess)
    return -1;
  const int ntiles = (d.n + kNC - 1) / kNC;
  const int need = (ntiles + kWG - 1) / kWG;
  const int grid = need < sms ? need : sms;
  if (grid <= 0) return 0;
  sei_lintt<ORD><<<grid, 128 * kWG, Dm::kSmem, (cudaStream_t)stream>>>(a);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

namespace sei {

int launchLintTransposed(int order, const DeviceArrays& d, float* trace, int traceOnly, int* status, int sms,
                         void* stream) {
#define SEI_LT_ARGS(o)                                                                                          \
  (const void*)&sei_tc_o##o::kvolt_op, (const void*)&sei_tc_o##o::kvolt_scale, (const void*)&sei_tc_o##o::krtt_op, \
      (const void*)&sei_tc_o##o::krtt_scale, (const void*)&sei_tc_o##o::krtt_tsc, (const void*)&sei_tc_o##o::kinvm
  switch (order) {
    case 4:
      return launchLintt<4>(d, trace, traceOnly, status, sms, stream, SEI_LT_ARGS(4));
    case 5:
      return launchLintt<5>(d, trace, traceOnly, status, sms, stream, SEI_LT_ARGS(5));
    case 6:
      return launchLintt<6>(d, trace, traceOnly, status, sms, stream, SEI_LT_ARGS(6));
    default:
      return -1;
  }
#undef SEI_LT_ARGS
}

}  // namespace sei
