// Blackwell (sm_103a) tensor-core primitives: tcgen05 MMA with TMEM accumulators.
//
// Operand layout in shared memory: K-major, no swizzle.  The tile is cut into "core matrices"
// of 8 rows x 16 bytes (8 rows x 4 tf32), each stored as 128 contiguous bytes (row r at r*16).
// Core matrix (row group g, K chunk j) of a tile with KC chunks along K sits at byte offset
// (g * KC + j) * 128, i.e. the leading byte offset (next K chunk) is 128 and the stride byte
// offset (next 8-row group) is KC * 128.  One kind::tf32 MMA consumes K = 8 = 2 chunks, so
// the descriptor start address advances by 256 bytes per K step.
#pragma once
#include <cstdint>

namespace sei_tc {

// Byte offset of element (row, k) in a K-major no-swizzle tile with kc chunks of 4 floats along K.
__host__ __device__ __forceinline__ uint32_t kmajorOffset(int row, int k, int kc) {
  return (uint32_t)(((row >> 3) * kc + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor (version 1 = sm_100 family), no swizzle.
__device__ __forceinline__ uint64_t smemDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, absolute LBO mode, layout type 0 = no swizzle
}

// Instruction descriptor of kind::tf32: F32 accumulator, TF32 A and B, both K-major.
__host__ __device__ constexpr uint32_t idescTf32(int M, int N) {
  return (1u << 4)                    // D format F32
         | (2u << 7)                  // A format TF32
         | (2u << 10)                 // B format TF32
         | ((uint32_t)(N >> 3) << 17) // N / 8
         | ((uint32_t)(M >> 4) << 24);// M / 16
}

// Instruction descriptor of kind::f16: F32 accumulator, FP16 A and B, both K-major (K = 16 per MMA).
__host__ __device__ constexpr uint32_t idescF16(int M, int N) {
  return (1u << 4)                     // D format F32
         | ((uint32_t)(N >> 3) << 17)  // N / 8 (A, B format 0 = F16)
         | ((uint32_t)(M >> 4) << 24); // M / 16
}

// kind::f16 with the operand majors given: bMN = 1 reads B MN-major (N contiguous in 16-byte
// rows of a core matrix) instead of K-major.
__host__ __device__ constexpr uint32_t idescF16Major(int M, int N, int aMN, int bMN) {
  return idescF16(M, N) | ((uint32_t)(aMN & 1) << 15) | ((uint32_t)(bMN & 1) << 16);
}

// Byte offset of 16-bit element (row, k) in a K-major no-swizzle tile with kc chunks of 8 along K.
__host__ __device__ __forceinline__ uint32_t kmajorOffset16(int row, int k, int kc) {
  return (uint32_t)(((row >> 3) * kc + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 16 (fp16).
__device__ __forceinline__ void mmaSSf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accum)
      : "memory");
}

// Bulk (non-tensor) TMA copy global -> shared, completing tx bytes on the mbarrier.
__device__ __forceinline__ void mbarExpectTx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smemAddr(mbar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulkCopyG2S(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smemAddr(dst)),
               "l"(src), "r"(bytes), "r"(smemAddr(mbar))
               : "memory");
}

// Bulk (non-tensor) TMA copy shared -> global in the calling thread's bulk group; then
// bulkCommit() and bulkWaitRead() before the shared source is overwritten or the CTA exits.
__device__ __forceinline__ void bulkCopyS2G(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smemAddr(src)), "r"(bytes)
               : "memory");
}
// The same with an element-wise f32 add into global memory (dst[i] += src[i], performed in L2).
__device__ __forceinline__ void bulkReduceAddS2G(float* dst, const float* src, uint32_t bytes) {
  asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;\n" ::"l"(dst),
               "r"(smemAddr(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulkCommit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulkWaitRead() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }

// Bulk prefetch of [p, p + bytes) into L2 (p 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void prefetchL2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}

// One full warp allocates ncols TMEM columns; the address is written to *slot (shared).
__device__ __forceinline__ void tmemAlloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 8 (tf32).
__device__ __forceinline__ void mmaSS(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accum)
      : "memory");
}

// Arrives on the mbarrier once all previously issued MMAs of this thread have completed.
__device__ __forceinline__ void mmaCommit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smemAddr(mbar))
               : "memory");
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Makes generic-proxy shared-memory writes visible to the tensor-core (async) proxy.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbarInit(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Waits for the phase with the given parity; gives up after maxPolls polls and returns false.
__device__ __forceinline__ bool mbarWait(uint64_t* mbar, uint32_t parity, uint32_t maxPolls) {
  const uint32_t a = smemAddr(mbar);
  for (uint32_t i = 0; i < maxPolls; ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive 32-bit TMEM columns of this thread's lane (warp w reads lanes 32 (w % 4) ...).
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmemLoadWait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// 8 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmemLoad8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// .16x64b shape, for M = 64 accumulators (rows on lanes 0..15 of each warp's quarter): thread t
// of the warp receives lane base + (t >> 2) + 8 (t & 1), and register r holds column
// 2 r + ((t >> 1) & 1) of it; x32 covers 64 columns, x4 covers 8.
__device__ __forceinline__ void tmemLoad16x64b32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.16x64b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmemLoad16x64b4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.16x64b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

// Writes 16 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmemStore16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tmemStoreWait() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

// Power-of-two scaling without ldexpf/frexpf: the binary exponent e of m > 0 in the frexp
// convention (m = f 2^e, f in [0.5, 1)) from its bits, clamped to [-125, 126] (a zero or
// subnormal m gives -125), and 2^e as a float built from the exponent field.
__device__ __forceinline__ int pow2Exp(float m) {
  const int e = (int)((__float_as_uint(m) >> 23) & 0xFF) - 126;
  return e < -125 ? -125 : (e > 126 ? 126 : e);
}
__device__ __forceinline__ float pow2(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }

// Splits x into a TF32-exact high part (low 13 mantissa bits cleared) and the remainder.
__device__ __forceinline__ void splitTf32(float x, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

}  // namespace sei_tc
