// Stage 1 on the 5th-generation tensor cores (sm_103a): the masked_logdot
// score of every (query, edge) pair (core.ml:187-197, Glv.masked_logdot,
// linear_c.c:465-539) as one fused tcgen05 contraction per tile.
//
// The query side of masked_logdot is the full query evolved by start_pend,
// so its value at a site depends only on the site's character.  With
//   T[e][c][s] = log(sum_r sum_k qe_c[r][k] snode_e[s][r][k])
// and the supernode exponents ex[e][s], the score of (q, e) is
//   sum_{s in q, code c primary} T[e][c][s]  - n_q log R
//   + ln 2 (sum_{s informative in q} ex[e][s]),
// ambiguity characters added afterwards by k_s1_scores.  Per tile of 128
// edges (MMA M, operand A) x N <= 256 queries (MMA N, operand B):
//   * A: T split into three bf16 terms (hi + mid + lo keep 24 mantissa
//     bits), layout [plane][code][edge][site], and the exponents rebased per
//     edge (ex - base_e) as two exact bf16 digits (256 hi, lo), layout
//     [digit][edge][site]; loaded by TMA (cp.async.bulk.tensor, 64-byte
//     swizzle) in chunks of 32 sites.
//   * B: the queries' one-hot rows for one code (1.0 where the site holds
//     that primary code) or the informative mask, generated in shared memory
//     from the per-site classes by four warps (never stored in HBM).
//   * D: two FP32 accumulators in TMEM, C (the T sums; three MMAs per code
//     and K step, hi/mid/lo) and X (the exponent digits; the integer sums
//     stay exact while every partial sum is below 2^24, which the table
//     kernel checks per edge), 256 columns each.
// Warp roles: warp 0 issues the TMA loads, warp 1 the MMAs (one thread),
// warps 2-5 build the B tiles and then read TMEM for the epilogue, which
// writes per (query, edge) the pair (C as FP32, the exact total exponent sum
// as int32); the ranking forms the score from it as an exact pair of
// floats (s1_pair_df), so no FP64 arithmetic -- slow on this part -- sits
// in the tile loop or the ranking.  The
// query tile width N (a multiple of 16, up to 256) is chosen per launch to
// fill the SMs' last wave.  Stages are handed over through mbarriers; every
// wait is bounded and a timeout records where it happened and returns.
#pragma once
#include <cuda.h>

#include "tc.cuh"

namespace pgb {
namespace s1 {

constexpr int kSites = 32;                         // sites per K chunk: 64 B of bf16, one swizzle row
constexpr int kEdges = 128;                        // MMA M
constexpr int kQueries = 256;                      // MMA N at most (the launch's N: MmaCtx::nq)
constexpr int kStages = 5;
constexpr int kATile = kEdges * kSites * 2;        // one plane: 8 KB
constexpr int kABytes = 3 * kATile;                // hi / mid / lo planes (the exponent unit uses two)
constexpr int kBBytes = kQueries * kSites * 2;     // 16 KB
constexpr int kStageBytes = kABytes + kBBytes;     // 40 KB
constexpr int kThreads = 192;
constexpr int kGen = 128;                          // B-tile / epilogue threads (warps 2-5)
constexpr uint32_t kTmemCols = 512;                // C: [0, 256), X: [256, 512)
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 1024 + 256 + kQueries * sizeof(int);
constexpr int kMaxExpDigitSum = 1 << 24;           // exact FP32 integer range of the X accumulator
constexpr double kLn2d = 0.69314718055994530942;

// kind::f16 instruction descriptor: D F32, A and B BF16, both K-major,
// M = 128, N = nq.
__host__ __device__ constexpr uint32_t idesc_bf16(int nq) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nq >> 3) << 17) | ((uint32_t)(kEdges >> 4) << 24);
}

// Shared-memory descriptor of a K-major operand tile in the 64-byte swizzle
// layout: rows of 64 B, 8-row groups 512 B apart (stride byte offset), the
// fixed 0b001 at bits 46-48, layout type 4 (SWIZZLE_64B) at bits 61-63.
// The tiles are 1024-byte aligned, so a K step of 16 elements (32 B) within
// the row is a plain start-address offset.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3ffffu) >> 4) | (1ull << 16) | ((uint64_t)(512 >> 4) << 32) | (1ull << 46) |
         (4ull << 61);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
      "}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
      "%6}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(tc::smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(tc::smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

struct MmaCtx {
  int S, n_chunks, prim, n_edges, Q, n_qtiles, Sc;
  int nq;                // queries per tile (MMA N): a multiple of 16, 16..256
  const uint8_t *qc;     // [>= n_qtiles * nq][Sc] site classes: 0 not informative, c + 1 primary code c, 255 other
  const int *qlen;       // informative sites per query
  const int *qstatus;
  const int *ebase;      // per-edge exponent base
  int2 *pairs;           // [Q][n_edges]: (C as float bits, total exponent sum)
  int *err;              // [0] flag, [1] role, [2] unit, [3] block
};

// The stage-1 score of a (C, exponent sum x) pair, C - n log R + ln 2 x
// (masked_logdot's float part and the exponent term of Glv.masked_logdot),
// as an unevaluated sum hi + lo of two floats: exact products and sums
// (Dekker / Knuth error-free transformations on FMA) keep about 44 bits,
// and FP32 runs at many times FP64's rate on this part.  hi + lo is exact in
// FP64, which is the score pgb_queries_stage1 returns; the ranking compares
// the pairs, normalised so that |lo| <= ulp(hi) / 2, by (hi, lo).
struct QConst {
  float hi, lo;  // -n log R as a float pair
};
__device__ __forceinline__ QConst s1_qconst(int qlen, double log_nrates) {
  const double v = -(double)(float)qlen * log_nrates;
  QConst c;
  c.hi = (float)v;
  c.lo = (float)(v - (double)c.hi);
  return c;
}
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ float2 s1_pair_df(int2 p, QConst qc) {
  constexpr float kL2H = 0.693147182464599609375f;      // ln 2 rounded to float
  constexpr float kL2L = -1.904654299957768e-09f;       // ln 2 - kL2H
  const float c = __int_as_float(p.x);
  const float xh = (float)p.y;                           // x within 64 of xh
  const float xl = (float)(p.y - (int)xh);               // exact
  const float ph = kL2H * xh;
  float pl = fmaf(kL2H, xh, -ph);                        // exact error of ph
  pl = fmaf(kL2L, xh, fmaf(kL2H, xl, pl));
  float s1, e1, s2, e2;
  two_sum(c, ph, s1, e1);
  two_sum(s1, qc.hi, s2, e2);
  const float t = e1 + e2 + pl + qc.lo;
  float hi, lo;
  two_sum(s2, t, hi, lo);
  return make_float2(hi, lo);
}
__device__ __forceinline__ double s1_pair_score(int2 p, QConst qc) {
  const float2 v = s1_pair_df(p, qc);
  return (double)v.x + (double)v.y;
}
// Order-preserving 64-bit key of the pair: hi's order bits, then lo's (NaN
// lowest).
__device__ __forceinline__ uint32_t s1_fkey(float v) {
  const uint32_t b = __float_as_uint(v);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long s1_pair_key(int2 p, QConst qc) {
  const float2 v = s1_pair_df(p, qc);
  if (isnan(v.x) || isnan(v.y)) return 0ull;
  return ((unsigned long long)s1_fkey(v.x) << 32) | s1_fkey(v.y);
}

// Bounded wait; gives up when another role aborted or after the poll limit
// (then it aborts the block).
__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  for (int i = 0; i < tc::kWaitLimit; i++) {
    if (tc::bar_try_wait(bar, parity)) return true;
    if ((i & 255) == 255 && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

__device__ __forceinline__ void record(const MmaCtx &c, int role, int unit) {
  if (atomicCAS(c.err, 0, 1) == 0) {
    c.err[1] = role;
    c.err[2] = unit;
    c.err[3] = blockIdx.x;
  }
}

// One B row (a query, 32 sites) of the one-hot / mask tile: 1.0 (bf16
// 0x3F80) where the site's class matches `cls` (0: any informative class),
// in the 64-byte swizzle layout (16-byte chunk j of row r at j ^ ((r >> 1) & 3)).
__device__ __forceinline__ void write_b_row(uint8_t *tile, int r, const uint32_t (&w)[8], uint32_t cls) {
  const uint32_t pat = cls * 0x01010101u;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    uint32_t m0 = cls ? __vcmpeq4(w[2 * j], pat) : __vcmpne4(w[2 * j], 0u);
    uint32_t m1 = cls ? __vcmpeq4(w[2 * j + 1], pat) : __vcmpne4(w[2 * j + 1], 0u);
    uint4 v;
    v.x = __byte_perm(m0, 0, 0x1100) & 0x3F803F80u;
    v.y = __byte_perm(m0, 0, 0x3322) & 0x3F803F80u;
    v.z = __byte_perm(m1, 0, 0x1100) & 0x3F803F80u;
    v.w = __byte_perm(m1, 0, 0x3322) & 0x3F803F80u;
    *reinterpret_cast<uint4 *>(tile + r * 64 + ((j ^ ((r >> 1) & 3)) << 4)) = v;
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    k_s1_mma(const __grid_constant__ CUtensorMap tmT, const __grid_constant__ CUtensorMap tmX, MmaCtx c) {
  extern __shared__ uint8_t s1_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(s1_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(base + (size_t)kStages * kStageBytes);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  // per query column: n_q, or -1 when no score is written
  int *q_n = reinterpret_cast<int *>(base + (size_t)kStages * kStageBytes + 256);
  const uint32_t idesc = idesc_bf16(c.nq);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int etile = blockIdx.x / c.n_qtiles, qtile = blockIdx.x - etile * c.n_qtiles;
  const int per_chunk = c.prim + 1;  // prim code units, then the exponent unit
  const int U = c.n_chunks * per_chunk;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; i++) {
      tc::bar_init(&full[i], 1 + kGen);
      tc::bar_init(&empty[i], 1);
    }
    tc::bar_init(done, 1);
    *abort_flag = 0;
  }
  if (warp == 0) tc::tmem_alloc(tmem_slot, kTmemCols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // ---- TMA producer ----
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmT)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmX)) : "memory");
      int issued = 0;
      for (int u = 0; u < U; u++) {
        const int s = u % kStages;
        if (!wait_bar(&empty[s], ((u / kStages) & 1) ^ 1, abort_flag)) {
          record(c, 1, u);
          break;
        }
        const int chunk = u / per_chunk, j = u - chunk * per_chunk;
        const uint32_t dst = tc::smem_addr(base + (size_t)s * kStageBytes);
        if (j < c.prim) {
          arrive_expect_tx(&full[s], kABytes);
          tma_load_4d(dst, &tmT, &full[s], chunk * kSites, etile * kEdges, j, 0);
        } else {
          arrive_expect_tx(&full[s], 2 * kATile);
          tma_load_3d(dst, &tmX, &full[s], chunk * kSites, etile * kEdges, 0);
        }
        issued = u + 1;
      }
      // the copies in flight land before the block exits (bounded)
      for (int u = issued - 1; u >= 0 && u >= issued - kStages; u--) {
        volatile int never = 0;
        wait_bar(&full[u % kStages], (u / kStages) & 1, &never);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---- MMA issuer ----
      uint32_t acc_c = 0, acc_x = 0;
      for (int u = 0; u < U; u++) {
        const int s = u % kStages;
        if (!wait_bar(&full[s], (u / kStages) & 1, abort_flag)) {
          record(c, 2, u);
          break;
        }
        tc::fence_after();
        const uint32_t a = tc::smem_addr(base + (size_t)s * kStageBytes), b = a + kABytes;
        const int j = u % per_chunk;
        if (j < c.prim) {
#pragma unroll
          for (int p = 0; p < 3; p++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
              mma_bf16(tmem, sdesc_sw64(a + p * kATile + k * 32), sdesc_sw64(b + k * 32), idesc, acc_c);
              acc_c = 1;
            }
        } else {
#pragma unroll
          for (int p = 0; p < 2; p++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
              mma_bf16(tmem + 256, sdesc_sw64(a + p * kATile + k * 32), sdesc_sw64(b + k * 32), idesc, acc_x);
              acc_x = 1;
            }
        }
        tc::commit(&empty[s]);  // the stage is free once these MMAs have read it
      }
      tc::commit(done);
    }
  } else {
    // ---- B tiles: two query rows per thread ----
    const int g = threadIdx.x - 64;
    const int r0 = g, r1 = g + kGen;
    const bool has_r1 = r1 < c.nq;
#pragma unroll
    for (int i = 0; i < 2; i++) {  // the epilogue's per-query terms
      const int r = i ? r1 : r0, q = qtile * c.nq + r;
      if (r < c.nq) q_n[r] = (q < c.Q && c.qstatus[q] == PGB_Q_OK) ? c.qlen[q] : -1;
    }
    const uint8_t *row0 = c.qc + (size_t)(qtile * c.nq + r0) * c.Sc;
    const uint8_t *row1 = c.qc + (size_t)(qtile * c.nq + (has_r1 ? r1 : r0)) * c.Sc;
    bool ok = true;
    // the next chunk's site classes are loaded while this chunk's tiles are built
    uint4 nx[4];
    auto load_chunk = [&](int chunk) {
      const uint4 *p0 = reinterpret_cast<const uint4 *>(row0 + chunk * kSites);
      const uint4 *p1 = reinterpret_cast<const uint4 *>(row1 + chunk * kSites);
      nx[0] = __ldg(p0); nx[1] = __ldg(p0 + 1); nx[2] = __ldg(p1); nx[3] = __ldg(p1 + 1);
    };
    load_chunk(0);
    for (int chunk = 0; chunk < c.n_chunks && ok; chunk++) {
      uint32_t w0[8], w1[8];
      w0[0] = nx[0].x; w0[1] = nx[0].y; w0[2] = nx[0].z; w0[3] = nx[0].w;
      w0[4] = nx[1].x; w0[5] = nx[1].y; w0[6] = nx[1].z; w0[7] = nx[1].w;
      w1[0] = nx[2].x; w1[1] = nx[2].y; w1[2] = nx[2].z; w1[3] = nx[2].w;
      w1[4] = nx[3].x; w1[5] = nx[3].y; w1[6] = nx[3].z; w1[7] = nx[3].w;
      if (chunk + 1 < c.n_chunks) load_chunk(chunk + 1);
      for (int j = 0; j < per_chunk; j++) {
        const int u = chunk * per_chunk + j, s = u % kStages;
        if (!wait_bar(&empty[s], ((u / kStages) & 1) ^ 1, abort_flag)) {
          record(c, 3, u);
          ok = false;
          break;
        }
        uint8_t *tile = base + (size_t)s * kStageBytes + kABytes;
        const uint32_t cls = j < c.prim ? (uint32_t)(j + 1) : 0u;
        write_b_row(tile, r0, w0, cls);
        if (has_r1) write_b_row(tile, r1, w1, cls);
        tc::fence_async_smem();
        arrive(&full[s]);
      }
    }
    // ---- epilogue: TMEM lane = edge, column = query ----
    asm volatile("bar.sync 1, %0;" ::"n"(kGen) : "memory");  // the per-query terms are in place
    if (wait_bar(done, 0, abort_flag) && !*abort_flag) {
      tc::fence_after();
      const int quarter = warp & 3;  // the TMEM lanes this warp may read
      const int e = etile * kEdges + quarter * 32 + lane;
      const bool e_ok = e < c.n_edges;
      const int eb = e_ok ? c.ebase[e] : 0;
      const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
      int2 *out = c.pairs + (size_t)qtile * c.nq * c.n_edges + e;
      for (int c0 = 0; c0 < c.nq; c0 += 16) {
        float vc[16], vx[16];
        tc::ld16(lane_addr + c0, vc);
        tc::ld16(lane_addr + 256 + c0, vx);
        tc::ld_wait();
        tc::pin(vc);
        tc::pin(vx);
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int n = q_n[c0 + i];
          if (e_ok && n >= 0)  // vx holds an exact integer; add back n_q times the edge's base
            __stcs(out + (size_t)(c0 + i) * c.n_edges, make_int2(__float_as_int(vc[i]), __float2int_rn(vx[i]) + eb * n));
        }
      }
    } else {
      record(c, 4, U);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

// Per-site classes of the loaded queries for the B tiles: 0 not informative
// (gaps, padding, rows of failed queries), c + 1 for primary code c, 255 for
// an informative ambiguity character.  [rows][Sc], rows >= Q + 256.
__global__ void k_s1_qclass(int Q, int S, int Sc, int prim, const uint8_t *__restrict__ qcode,
                            const uint8_t *__restrict__ informative, const int *__restrict__ qstatus, uint8_t *qc) {
  const int q = blockIdx.x;
  const bool ok = q < Q && qstatus[q] == PGB_Q_OK;
  for (int s = threadIdx.x; s < Sc; s += blockDim.x) {
    uint8_t v = 0;
    if (ok && s < S) {
      const int code = qcode[(size_t)q * S + s];
      if (code != kBadCode && informative[code]) v = code < prim ? (uint8_t)(code + 1) : (uint8_t)255;
    }
    qc[(size_t)q * Sc + s] = v;
  }
}

__device__ __forceinline__ long long block_sum_ll(long long v, long long *sh) {
  v = warp_sum_ll(v);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  long long t = 0;
  for (int i = 0; i < nw; i++) t += sh[i];
  return t;
}

}  // namespace s1
}  // namespace pgb
