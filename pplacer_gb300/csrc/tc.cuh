// 5th-generation tensor core (tcgen05) building blocks for the 20-state
// evolve, sm_103a: operand tiles in shared memory (no swizzle, K-major),
// accumulators in tensor memory (TMEM), completion through an mbarrier.
//
// The evolve dst[s][i] = sum_j M[i][j] src[s][j] of pplacer's
// Gmix_model.evolve_into / gemmish (pplacer_src/gmix_model.ml:308-315,
// linear_c.c:29-90) is a GEMM with the sites as rows: A = the sites' state
// vectors [128 sites x K], B = the matrices' rows [N x K] (K-major, as
// stored), D = A B^T in TMEM (lane = site, column = output row).
//
// Precision: each FP32 operand x is split into hi = x rounded to TF32 and
// lo = x - hi (exact), and D accumulates hi*hi + hi*lo + lo*hi in FP32; the
// dropped lo*lo term and the TF32 rounding of lo are ~2^-22 relative, the
// order of FP32 arithmetic.
#pragma once
#include <stdint.h>

namespace pgb {
namespace tc {

constexpr int kKPad = 24;                        // states padded to three 8-element TF32 steps
constexpr int kGroupFloats = kKPad * 8;          // one 8-row group: 6 core matrices of 8 rows x 16 B
constexpr uint32_t kLBO = 128;                   // bytes between core matrices adjacent in K
constexpr uint32_t kSBO = kGroupFloats * 4;      // bytes between 8-row groups (768)
constexpr uint32_t kKStepBytes = 2 * kLBO;       // one 8-element K step = two core matrices
constexpr int kTileRows = 128;                   // sites per MMA (M)
constexpr int kTileFloats = kTileRows * kKPad;   // [128 x 24] operand tile

// Float offset of element (row, k) in a tile: row groups of 8 rows, each a
// run of 8 x 16 B core matrices along K.
__host__ __device__ __forceinline__ int off(int row, int k) {
  return (row >> 3) * kGroupFloats + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

// TF32 split: hi keeps the upper 10 mantissa bits (round to nearest, ties
// away), lo = x - hi exactly.
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
  hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
  lo = x - hi;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, the fixed 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of kind::tf32: D F32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t"
      "}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

// Arrive on the mbarrier once every tcgen05 operation issued so far by this
// thread has completed.
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t"
      "}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Non-blocking: has the phase of the given parity completed?
__device__ __forceinline__ bool bar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t"
      "}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of the given parity: false when it did not
// complete within the limit (the caller records an error and stops issuing).
constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
  for (int i = 0; i < kWaitLimit; i++)
    if (bar_try_wait(bar, parity)) return true;
  return false;
}

// Generic-proxy shared-memory writes become visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation: executed by one whole warp; the column base goes to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive 32-bit columns of the warp's 32 TMEM lanes (thread i gets
// lane base + i).  The values are valid after ld_wait().
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Ties loaded registers to a point after ld_wait(): the compiler cannot
// hoist their uses above it.
template <int N>
__device__ __forceinline__ void pin(float (&v)[N]) {
#pragma unroll
  for (int i = 0; i < N; i++) asm volatile("" : "+f"(v[i]));
}

// The same MMA with A in tensor memory: row m of the 128-row A tile in TMEM
// lane m, its K elements (TF32, one per 32-bit column) in consecutive
// columns from atmem; B from shared memory.
__device__ __forceinline__ void mma_tf32_ts(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t idesc,
                                            uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t"
      "}" ::"r"(dtmem),
      "r"(atmem), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

// 8 consecutive 32-bit columns of the warp's 32 TMEM lanes from registers
// (thread i writes lane base + i); complete after st_wait().
__device__ __forceinline__ void st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// A row of kKPad FP32 values (zero past the states) into TMEM as TF32 hi at
// columns [col_hi, col_hi + 24) and lo at [col_lo, col_lo + 24) of the
// thread's lane; taddr_lane = TMEM base with the warp's lane quarter.
__device__ __forceinline__ void st_split_row(uint32_t taddr_lane, uint32_t col_hi, uint32_t col_lo,
                                             const float (&v)[kKPad]) {
#pragma unroll
  for (int b = 0; b < kKPad / 8; b++) {
    float h[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; j++) split_tf32(v[8 * b + j], h[j], l[j]);
    st8(taddr_lane + col_hi + 8 * b, h);
    st8(taddr_lane + col_lo + 8 * b, l);
  }
}

// D[0:M, 0:N] (+)= A B^T over the three K steps of the padded states, with
// the 3xTF32 products: hi*hi, hi*lo, lo*hi, A in TMEM (columns a_hi, a_lo),
// B in shared memory; issued by one thread.
__device__ __forceinline__ void mma_3xtf32_ts(uint32_t dtmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                              uint32_t b_lo, uint32_t idesc) {
#pragma unroll
  for (int s = 0; s < kKPad / 8; s++) {
    const uint32_t o = s * kKStepBytes;
    mma_tf32_ts(dtmem, a_lo + 8 * s, sdesc(b_hi + o), idesc, s > 0 ? 1u : 0u);
    mma_tf32_ts(dtmem, a_hi + 8 * s, sdesc(b_lo + o), idesc, 1u);
    mma_tf32_ts(dtmem, a_hi + 8 * s, sdesc(b_hi + o), idesc, 1u);
  }
}

// Barrier of one team of kTeamThreads threads (named barrier id >= 1), and
// the same barrier as a vote: true when v is true in every thread.
constexpr int kTeamThreads = 128;
__device__ __forceinline__ void team_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(kTeamThreads) : "memory");
}
__device__ __forceinline__ bool team_and(int id, bool v) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t"
      "}"
      : "=r"(out)
      : "r"((uint32_t)v), "r"(id), "r"(kTeamThreads)
      : "memory");
  return out != 0;
}

// D[0:M, 0:N] (+)= A B^T over the three K steps of the padded states, with
// the 3xTF32 products: hi*hi, hi*lo, lo*hi.  a_hi, a_lo, b_hi, b_lo: shared
// addresses of the operand tiles; issued by one thread.
__device__ __forceinline__ void mma_3xtf32(uint32_t dtmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                           uint32_t b_lo, uint32_t idesc) {
#pragma unroll
  for (int s = 0; s < kKPad / 8; s++) {
    const uint32_t o = s * kKStepBytes;
    mma_tf32(dtmem, sdesc(a_lo + o), sdesc(b_hi + o), idesc, s > 0 ? 1u : 0u);
    mma_tf32(dtmem, sdesc(a_hi + o), sdesc(b_lo + o), idesc, 1u);
    mma_tf32(dtmem, sdesc(a_hi + o), sdesc(b_hi + o), idesc, 1u);
  }
}

}  // namespace tc
}  // namespace pgb
