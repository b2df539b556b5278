// Stage-2 trials of 20-state Gamma-mixture models on the tensor cores: one
// CTA of 128 threads per (query, location) optimisation (Three_tax.optimize,
// pplacer_src/three_tax.ml:48-83), the per-site evolves of the distal and
// proximal GLVs (Gmix_model.evolve_into, gmix_model.ml:308-315) as tcgen05
// MMAs.  Included by engine.cu inside its anonymous namespace, after
// trials.cuh.
//
// The operands are the GLVs in the eigenbasis of the rate matrix: with
// P(t) = X diag(exp(r lambda t)) X^-1, the evolved distal vector is
// P(t) D = X diag(e) (X^-1 D), and its t-derivatives put r lambda (or its
// square) beside e.  The A tiles are the rows X^-1 D (darr_e / parr_e, built
// once per tree), the B tiles the rows of X scaled by those factors, so a
// new branch length costs one cheap B-tile rewrite per rate instead of
// re-forming P.
//
// One evaluation at (pend, dist):
//   thread 0: optimiser -> next point                      | barrier
//   all: exp factors of the three lengths                  | barrier
//   query tables: the statd-weighted evolved query vectors of every
//        character code (and d/dpend, d2/dpend2) for every rate, one MMA group
//        per 128 rows (X rows scaled by the pendant factors) x Lt (the codes'
//        vectors in the eigenbasis)                         | barriers
//   per rate r:
//     all: B tiles of rate r -- X rows scaled by e, r lambda e, (r lambda)^2 e
//          at dist (distal) and cut - dist (proximal), TF32 hi / lo
//     per chunk of 128 sites:
//       all: the chunk's darr_e / parr_e rows (loaded during the previous
//            chunk's MMAs) split into TF32 hi / lo A tiles         | barrier
//       thread 0: 2 x 9 MMAs (3 K steps x 3 products) into TMEM columns
//                 [0, 64) (distal) and [64, 128) (proximal); commit
//       all: load the next chunk's rows; wait for the MMAs; each thread reads
//            its site's TMEM lane and adds the rate's site likelihood (and
//            derivatives) into the site's shared accumulators       | barrier
//   all: per-site (mantissa, exponent) products and derivative sums, CTA
//        reduction                                                  | barrier
// Value-only evaluations use N = 32 (the P rows only).  Every wait on the
// MMA completion is bounded; on a timeout the kernel records the error, stops
// issuing, waits once more (bounded) and frees its TMEM.

constexpr int kTcThreads = 128;
constexpr int kTcK = 20;
constexpr int kTcNDer = 64;     // B rows with derivatives: P, dP, d2P (3 x 20) + 4 zero rows
constexpr int kTcNVal = 32;     // B rows of a value-only evaluation: P (20) + 12 rows not read
constexpr int kTcCols = 128;    // TMEM columns per CTA: distal [0, 64), proximal [64, 128)
constexpr int kTcXs = kTcK + 1;  // padded row stride of X and Xit (bank spread)
constexpr int kTcZs = kTcK + 1;  // padded row stride of the query-vector tables
constexpr int kTcMaxRates = 4;   // query-table rows 3 x 4 x 20 fit two 128-row MMA tiles
static_assert(pgb::kMaxCodes <= 32, "the query-vector table GEMM has N = 32 codes");

struct TcSmem {
  float *a_dh, *a_dl, *a_xh, *a_xl;  // A tiles [128 x 24]: distal / proximal rows, hi / lo
  float *b_dh, *b_dl, *b_xh, *b_xl;  // B tiles [64 x 24]
  float *acc;                         // [6][cap] per-site sums over rates
  float *Z;                           // [3][NM][zcodes][kTcZs]: query vectors and d/dpend, d2/dpend2
  float *X;                           // [K][kTcXs]
  float *E, *Em1, *Lr;                // [3][NM][K], [3][NM][K], [NM][K]
  float *F;                           // [2][3][NM][K]: (r lambda)^m exp(r lambda t_g), the B-tile scales
  float *lv, *statd;
  float *red;                         // [4][8]
  int *redi;                          // [4]
  uint16_t *col;                      // [cap] alignment columns of the query's sites
  uint8_t *code;                      // [cap]
  Ctrl *ctrl;
  Optimiser *opt;
  TrialRes *res;  // a finished trial's result, read by every thread
  uint64_t *bar;
  uint32_t *tbase;
};

// zcodes: the character codes the query tables hold (the primary states,
// or every code when a query has ambiguity characters)
__host__ __device__ inline size_t tc_trial_smem_bytes(int cap, int NM, int ncode, int zcodes) {
  const int K = kTcK;
  size_t b = 4 * align16((size_t)pgb::tc::kTileFloats * 4) + 4 * align16((size_t)kTcNDer * pgb::tc::kKPad * 4);
  b += align16((size_t)6 * cap * 4);
  b += align16((size_t)3 * NM * zcodes * kTcZs * 4);
  b += align16((size_t)K * kTcXs * 4);
  b += 2 * align16((size_t)3 * NM * K * 4) + align16((size_t)NM * K * 4) + align16((size_t)6 * NM * K * 4);
  b += align16((size_t)ncode * K * 4) + align16((size_t)K * 4);
  b += align16(4 * 8 * 4) + align16(4 * 4);
  b += align16((size_t)cap * 2) + align16((size_t)cap);
  b += align16(sizeof(Ctrl)) + align16(sizeof(Optimiser)) + align16(sizeof(TrialRes)) + 16 + 16;
  return b + 1024;  // base alignment of the operand tiles
}

__device__ inline TcSmem tc_carve(char *base, int cap, int NM, int ncode, int zcodes) {
  const int K = kTcK;
  TcSmem s;
  char *p = (char *)(((uintptr_t)base + 1023) & ~(uintptr_t)1023);
  auto take = [&](size_t bytes) { char *r = p; p += align16(bytes); return r; };
  const size_t at = (size_t)pgb::tc::kTileFloats * 4, bt = (size_t)kTcNDer * pgb::tc::kKPad * 4;
  s.a_dh = (float *)take(at); s.a_dl = (float *)take(at); s.a_xh = (float *)take(at); s.a_xl = (float *)take(at);
  s.b_dh = (float *)take(bt); s.b_dl = (float *)take(bt); s.b_xh = (float *)take(bt); s.b_xl = (float *)take(bt);
  s.acc = (float *)take((size_t)6 * cap * 4);
  s.Z = (float *)take((size_t)3 * NM * zcodes * kTcZs * 4);
  s.X = (float *)take((size_t)K * kTcXs * 4);
  s.E = (float *)take((size_t)3 * NM * K * 4);
  s.Em1 = (float *)take((size_t)3 * NM * K * 4);
  s.Lr = (float *)take((size_t)NM * K * 4);
  s.F = (float *)take((size_t)6 * NM * K * 4);
  s.lv = (float *)take((size_t)ncode * K * 4);
  s.statd = (float *)take((size_t)K * 4);
  s.red = (float *)take(4 * 8 * 4);
  s.redi = (int *)take(4 * 4);
  s.col = (uint16_t *)take((size_t)cap * 2);
  s.code = (uint8_t *)take((size_t)cap);
  s.ctrl = (Ctrl *)take(sizeof(Ctrl));
  s.opt = (Optimiser *)take(sizeof(Optimiser));
  s.res = (TrialRes *)take(sizeof(TrialRes));
  s.bar = (uint64_t *)take(16);
  s.tbase = (uint32_t *)take(16);
  return s;
}

// float4 of row `row`, columns k .. k + 3, as TF32 hi / lo into two tiles
__device__ __forceinline__ void tc_store_split(float *hi, float *lo, int row, int k, float4 v) {
  float4 h, l;
  pgb::tc::split_tf32(v.x, h.x, l.x);
  pgb::tc::split_tf32(v.y, h.y, l.y);
  pgb::tc::split_tf32(v.z, h.z, l.z);
  pgb::tc::split_tf32(v.w, h.w, l.w);
  *reinterpret_cast<float4 *>(hi + pgb::tc::off(row, k)) = h;
  *reinterpret_cast<float4 *>(lo + pgb::tc::off(row, k)) = l;
}

// Query tables of every rate on the tensor cores: rows rho = (m * NM + r) *
// 20 + i (m = 0: value, 1, 2: d/dpend, d2/dpend2) of A = X[i][.] * f(.), f
// = expm1(r lambda pend), r lambda e, (r lambda)^2 e; times Lt^T (the codes'
// likelihood vectors in the eigenbasis, written into the distal B tiles,
// which are free until the rate's B tiles) gives sum_k X[i][k] f_k Lt[code][k],
// so that Z = statd_i * (lv[code][i] + that) for m = 0 (P = I + X diag(expm1)
// X^-1) and statd_i * that for the derivatives.  Rows 0..127 go through
// (a_dh, a_dl) into TMEM columns [0, 32), rows 128.. through (a_xh, a_xl)
// into [32, 64).  Returns false when the completion wait timed out.
template <bool DER>
__device__ __forceinline__ bool tc_query_tables(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, int NM, int ncz,
                                                int nc, int zc, int tid, uint32_t &phase) {
  namespace T = pgb::tc;
  const int K = kTcK;
  const int rows = (DER ? 3 : 1) * NM * K;  // <= 240
  // B: the rows of Lt (codes), zero past the codes (rows 32..63 unused)
  for (int it = tid; it < 32 * (K / 4); it += kTcThreads) {
    const int row = it / (K / 4), k = (it - row * (K / 4)) * 4;
    const float4 v = row < nc ? *reinterpret_cast<const float4 *>(c.Lt + row * K + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    tc_store_split(sm.b_dh, sm.b_dl, row, k, v);
  }
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int rho = tid + h * T::kTileRows;
    if (rho < rows) {
      const int m = rho / (NM * K), r = (rho / K) % NM, i = rho % K;
      const float *x = sm.X + i * kTcXs, *lr = sm.Lr + r * K;
      const float *em = sm.Em1 + (2 * NM + r) * K, *e = sm.E + (2 * NM + r) * K;
#pragma unroll
      for (int k = 0; k < K; k += 4) {
        float v[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
          v[j] = x[k + j] * (m == 0 ? em[k + j] : (m == 1 ? lr[k + j] : lr[k + j] * lr[k + j]) * e[k + j]);
        tc_store_split(h == 0 ? sm.a_dh : sm.a_xh, h == 0 ? sm.a_dl : sm.a_xl, tid, k,
                       make_float4(v[0], v[1], v[2], v[3]));
      }
    }
  }
  T::fence_async_smem();
  __syncthreads();
  if (tid == 0) {
    T::fence_after();
    const uint32_t id = T::idesc_tf32(T::kTileRows, 32);
    T::mma_3xtf32(tmem, T::smem_addr(sm.a_dh), T::smem_addr(sm.a_dl), T::smem_addr(sm.b_dh), T::smem_addr(sm.b_dl),
                  id);
    if (rows > T::kTileRows)
      T::mma_3xtf32(tmem + 32, T::smem_addr(sm.a_xh), T::smem_addr(sm.a_xl), T::smem_addr(sm.b_dh),
                    T::smem_addr(sm.b_dl), id);
    T::commit(sm.bar);
  }
  const bool mine = T::bar_wait(sm.bar, phase);
  const bool ok = __syncthreads_and(mine ? 1 : 0) != 0;
  if (!ok && tid == 0 && c.tc_err && atomicCAS(c.tc_err, 0, 1) == 0) {
    int *d = c.tc_err;
    d[1] = blockIdx.x; d[2] = -1; d[3] = -1; d[4] = (int)phase; d[5] = mine;
    d[6] = T::bar_test(sm.bar, phase); d[7] = T::bar_test(sm.bar, phase ^ 1u);
    d[8] = (int)tmem; d[9] = (int)T::smem_addr(sm.a_dh); d[10] = (int)T::smem_addr(sm.bar);
    __threadfence();
  }
  phase ^= 1u;
  T::fence_after();
  if (!ok) return false;
  const uint32_t ta = tmem + ((uint32_t)(32 * (tid >> 5)) << 16);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int rho = tid + h * T::kTileRows;
    if (h == 1 && rows <= T::kTileRows) break;  // uniform
    float zv[32];
    {
      float t16[16];
      T::ld16(ta + 32 * h, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) zv[j] = t16[j];
      T::ld16(ta + 32 * h + 16, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) zv[16 + j] = t16[j];
    }
    T::ld_wait();
    T::pin(zv);
    if (rho < rows) {
      const int m = rho / (NM * K), i = rho % K;
      const float pi = sm.statd[i];
      float *z = sm.Z + (size_t)(rho / K) * zc * kTcZs + i;  // table (m, r), column i
#pragma unroll
      for (int code = 0; code < 32; code++)
        if (code < ncz) z[code * kTcZs] = pi * (m == 0 ? zv[code] + sm.lv[code * K + i] : zv[code]);
    }
  }
  T::fence_before();  // the next barrier orders these TMEM reads before the chunk MMAs
  return true;
}

// The B-tile scales of every rate, with the exp factors of the evaluation
// (published by the same barrier): F[g][m][r][k] = (r lambda_k)^m *
// exp(r lambda_k t_g), t_0 = dist, t_1 = cut - dist.
__device__ __forceinline__ void tc_scales(const TcSmem &sm, int NM, const Ctrl &ctl, int tid) {
  const int K = kTcK;
  for (int it = tid; it < 6 * NM * K; it += kTcThreads) {
    const int g = it / (3 * NM * K), m = (it / (NM * K)) % 3, rk = it % (NM * K);
    const float lr = sm.Lr[rk];
    const float e = expf(lr * (g == 0 ? ctl.dist : ctl.prox));
    sm.F[it] = (m == 0 ? 1.f : (m == 1 ? lr : lr * lr)) * e;
  }
}

// B tiles of rate r: row m * 20 + i, column k = X[i][k] * F[g][m][r][k]
// (distal tiles g = 0, proximal g = 1).  The previous MMAs have completed
// (their wait and barrier).
template <bool DER>
__device__ __forceinline__ void tc_btiles(const TcSmem &sm, int NM, int r, int tid) {
  const int K = kTcK;
  const int nrow = DER ? 3 * K : K;
  for (int it = tid; it < 2 * nrow * (K / 4); it += kTcThreads) {
    const int g = it / (nrow * (K / 4)), rem = it - g * nrow * (K / 4);
    const int n = rem / (K / 4), k = (rem - n * (K / 4)) * 4;
    const int m = n / K, i = n - m * K;
    const float *x = sm.X + i * kTcXs;
    const float4 f = *reinterpret_cast<const float4 *>(sm.F + ((g * 3 + m) * NM + r) * K + k);
    tc_store_split(g == 0 ? sm.b_dh : sm.b_xh, g == 0 ? sm.b_dl : sm.b_xl, n, k,
                   make_float4(x[k] * f.x, x[k + 1] * f.y, x[k + 2] * f.z, x[k + 3] * f.w));
  }
}

// The chunk's rows of rate r: darr / parr[node] at the sites' columns (zero
// past Sq).
struct TcRows {
  float4 d[5], x[5];
};
__device__ __forceinline__ void tc_load_rows(const TrialCtx &c, const TcSmem &sm, int node, int Sq, int r, int ch,
                                             int tid, TcRows &rw) {
  const int i = ch * pgb::tc::kTileRows + tid;
  if (i < Sq) {
    const long o = (((long)node * c.S + sm.col[i]) * c.RP + r) * kTcK;
    const float4 *dp = reinterpret_cast<const float4 *>(c.darr_e + o);
    const float4 *xp = reinterpret_cast<const float4 *>(c.parr_e + o);
#pragma unroll
    for (int k = 0; k < 5; k++) { rw.d[k] = __ldg(dp + k); rw.x[k] = __ldg(xp + k); }
  } else {
#pragma unroll
    for (int k = 0; k < 5; k++) rw.d[k] = rw.x[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// One rate of one chunk: MMAs, then the epilogue adds the rate's site
// likelihood and derivatives into the site's accumulators.  Returns false
// when the completion wait timed out.
template <bool DER>
__device__ __forceinline__ bool tc_chunk(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, int node, int Sq,
                                         int r, int ch, int nch, int cap, int tid, uint32_t &phase, TcRows &rw) {
  namespace T = pgb::tc;
  const int K = kTcK;
  // A tiles from the rows loaded earlier
#pragma unroll
  for (int k = 0; k < 5; k++) {
    tc_store_split(sm.a_dh, sm.a_dl, tid, 4 * k, rw.d[k]);
    tc_store_split(sm.a_xh, sm.a_xl, tid, 4 * k, rw.x[k]);
  }
  T::fence_async_smem();
  __syncthreads();
  if (tid == 0) {
    T::fence_after();
    const uint32_t id = T::idesc_tf32(T::kTileRows, DER ? kTcNDer : kTcNVal);
    T::mma_3xtf32(tmem, T::smem_addr(sm.a_dh), T::smem_addr(sm.a_dl), T::smem_addr(sm.b_dh),
                  T::smem_addr(sm.b_dl), id);
    T::mma_3xtf32(tmem + 64, T::smem_addr(sm.a_xh), T::smem_addr(sm.a_xl), T::smem_addr(sm.b_xh),
                  T::smem_addr(sm.b_xl), id);
    T::commit(sm.bar);
  }
  // the next chunk's rows (next rate's first chunk after the last) in flight
  // during the MMAs
  {
    int nr = r, nc2 = ch + 1;
    if (nc2 == nch) { nr = r + 1; nc2 = 0; }
    if (nr < c.RP) tc_load_rows(c, sm, node, Sq, nr, nc2, tid, rw);
  }
  const bool mine = T::bar_wait(sm.bar, phase);
  const bool ok = __syncthreads_and(mine ? 1 : 0) != 0;  // uniform over the CTA
  if (!ok && tid == 0 && c.tc_err && atomicCAS(c.tc_err, 0, 1) == 0) {
    // where the wait gave up: trial CTA, rate, chunk, phase and barrier state
    int *d = c.tc_err;
    d[1] = blockIdx.x; d[2] = r; d[3] = ch; d[4] = (int)phase; d[5] = mine;
    d[6] = T::bar_test(sm.bar, phase); d[7] = T::bar_test(sm.bar, phase ^ 1u);
    d[8] = (int)tmem; d[9] = (int)T::smem_addr(sm.a_dh); d[10] = (int)T::smem_addr(sm.bar);
    d[11] = Sq; d[12] = nch;
    __threadfence();
  }
  phase ^= 1u;
  T::fence_after();
  if (!ok) return false;
  const int w = tid >> 5;
  const uint32_t ta = tmem + ((uint32_t)(32 * w) << 16);
  const int i = ch * T::kTileRows + tid;
  const int code = i < Sq ? sm.code[i] : 0;
  const int NM = c.NM, zc = c.zcodes;
  const float *z = sm.Z + ((size_t)r * zc + code) * kTcZs;
  float u = 0.f, ud = 0.f, udd = 0.f, up = 0.f, upp = 0.f, upd = 0.f;
  if (DER) {
    float dv[64], xv[64];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      float t16[16];
      T::ld16(ta + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) dv[16 * b + j] = t16[j];
      T::ld16(ta + 64 + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) xv[16 * b + j] = t16[j];
    }
    T::ld_wait();
    T::pin(dv);
    T::pin(xv);
    const float *z1 = z + (size_t)NM * zc * kTcZs, *z2 = z1 + (size_t)NM * zc * kTcZs;
#pragma unroll
    for (int ii = 0; ii < K; ii++) {
      const float x = dv[ii], x1 = dv[K + ii], x2 = dv[2 * K + ii];
      const float y = xv[ii], y1 = xv[K + ii], y2 = xv[2 * K + ii];
      const float xy = x * y;
      const float aa = x1 * y - x * y1;
      const float bb = x2 * y - 2.f * x1 * y1 + x * y2;
      const float zz = z[ii], zz1 = z1[ii], zz2 = z2[ii];
      u = fmaf(zz, xy, u);
      ud = fmaf(zz, aa, ud);
      udd = fmaf(zz, bb, udd);
      up = fmaf(zz1, xy, up);
      upp = fmaf(zz2, xy, upp);
      upd = fmaf(zz1, aa, upd);
    }
  } else {
    float dv[32], xv[32];
#pragma unroll
    for (int b = 0; b < 2; b++) {
      float t16[16];
      T::ld16(ta + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) dv[16 * b + j] = t16[j];
      T::ld16(ta + 64 + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) xv[16 * b + j] = t16[j];
    }
    T::ld_wait();
    T::pin(dv);
    T::pin(xv);
#pragma unroll
    for (int ii = 0; ii < K; ii++) u = fmaf(z[ii], dv[ii] * xv[ii], u);
  }
  if (i < Sq) {
    float *a = sm.acc + i;
    if (r == 0) {
      a[0] = u;
      if (DER) { a[cap] = ud; a[2 * cap] = udd; a[3 * cap] = up; a[4 * cap] = upp; a[5 * cap] = upd; }
    } else {
      a[0] += u;
      if (DER) { a[cap] += ud; a[2 * cap] += udd; a[3 * cap] += up; a[4 * cap] += upp; a[5 * cap] += upd; }
    }
  }
  T::fence_before();
  __syncthreads();  // TMEM and the A tiles are free again
  return true;
}

// rows (node, site, rate) of darr and parr times X^-1 (FP64 accumulation)
__global__ void k_eigen_glvs(const float *__restrict__ darr, const float *__restrict__ parr,
                             const double *__restrict__ Xit, long rows, float *darr_e, float *parr_e) {
  constexpr int K = kTcK;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * rows; t += (long)gridDim.x * blockDim.x) {
    const bool prox = t >= rows;
    const long row = prox ? t - rows : t;
    const float *v = (prox ? parr : darr) + row * K;
    float *o = (prox ? parr_e : darr_e) + row * K;
    float x[K];
#pragma unroll
    for (int j = 0; j < K; j++) x[j] = v[j];
    for (int k = 0; k < K; k++) {
      double a = 0.0;
#pragma unroll
      for (int j = 0; j < K; j++) a += Xit[j * K + k] * (double)x[j];  // (X^-1)[k][j] = Xit[j][k]
      o[k] = (float)a;
    }
  }
}

// Per-CTA setup of the tensor-core trial kernels: model constants, the
// zero padding of the operand tiles (columns 20..23 of every tile, rows
// 60..63 of the B tiles, never written afterwards), TMEM columns and the
// mbarrier.  Returns the TMEM base.
__device__ __forceinline__ uint32_t tc_setup(const TrialCtx &c, const TcSmem &sm, int tid) {
  namespace T = pgb::tc;
  const int K = kTcK, NM = c.NM, nc = c.ncode;
  for (int it = tid; it < K * K; it += kTcThreads) {
    const int i = it / K, k = it - i * K;
    sm.X[i * kTcXs + k] = c.X[it];
  }
  for (int it = tid; it < nc * K; it += kTcThreads) sm.lv[it] = c.lvf[it];
  for (int it = tid; it < NM * K; it += kTcThreads) sm.Lr[it] = c.rates[it / K] * c.lam[it % K];
  if (tid < K) sm.statd[tid] = c.statd[tid];
  for (int it = tid; it < T::kTileFloats; it += kTcThreads) {
    sm.a_dh[it] = 0.f; sm.a_dl[it] = 0.f; sm.a_xh[it] = 0.f; sm.a_xl[it] = 0.f;
  }
  for (int it = tid; it < kTcNDer * T::kKPad; it += kTcThreads) {
    sm.b_dh[it] = 0.f; sm.b_dl[it] = 0.f; sm.b_xh[it] = 0.f; sm.b_xl[it] = 0.f;
  }
  __syncwarp();
  if ((tid >> 5) == 0) T::tmem_alloc(sm.tbase, kTcCols);
  if (tid == 0) T::bar_init(sm.bar, 1);
  T::fence_before();
  __syncthreads();
  T::fence_after();
  return *sm.tbase;
}

// After the last trial: a timed-out MMA group is waited for once more
// (bounded) and the TMEM columns are freed.
__device__ __forceinline__ void tc_teardown(const TcSmem &sm, uint32_t tmem, uint32_t phase, bool failed, int tid) {
  namespace T = pgb::tc;
  if (failed) T::bar_wait(sm.bar, phase ^ 1u);
  T::fence_before();
  __syncthreads();
  if ((tid >> 5) == 0) T::tmem_dealloc(tmem, kTcCols);
}

// One trial (Three_tax.optimize at one location, or its marginal
// likelihood) by the CTA; every thread returns the same result.  failed is
// set (in every thread) when an MMA completion wait timed out; the trial then
// reports status 1 and NaN.
__device__ TrialRes tc_trial(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, uint32_t &phase, bool &failed,
                             const TrialIn &tr, int tid) {
  namespace T = pgb::tc;
  const int K = kTcK;
  const int lane = tid & 31, warp = tid >> 5;
  const int NM = c.NM, nc = c.ncode, cap = c.cap, zc = c.zcodes;
  const int q = tr.q, node = tr.node;
  const int Sq = c.qlen[q];
  const int ncz = c.qamb[q] > 0 ? nc : c.prim;
  const int nch = (Sq + T::kTileRows - 1) / T::kTileRows;
  // ---- the query's sites and their exponent sum ----
  long long esum = 0;
  const long qo = (long)q * c.S;
  for (int i = tid; i < Sq; i += kTcThreads) {
    const int s = c.reind[qo + i];
    sm.col[i] = (uint16_t)s;
    sm.code[i] = c.mcode[qo + i];
    const long go = (long)node * c.S + s;
    esum += (long long)c.dexp[go] + (long long)c.pexp[go];
  }
  esum = warp_sum_ll(esum);
  __syncthreads();  // the previous trial's readers of red / res are done
  if (lane == 0) reinterpret_cast<long long *>(sm.red)[warp] = esum;
  __syncthreads();
  Optimiser &opt = *sm.opt;
  if (tid == 0) {
    long long etot = 0;
    for (int k = 0; k < kTcThreads / 32; k++) etot += reinterpret_cast<const long long *>(sm.red)[k];
    opt.optimizer = c.optimizer;
    opt.mode = c.mode;
    opt.cut = c.bl[node];
    opt.tol = tr.tol;
    opt.max_pend = c.max_pend;
    opt.start_pend = c.start_pend;
    opt.pend0 = tr.pend0;
    opt.dist0 = tr.dist0;
    opt.cst = kLn2 * (double)etot - (double)(float)Sq * c.log_nrates;
    opt.n_evals = 0;
    opt.seeded = tr.seeded != 0;
    opt.seed = tr.seed;
    if (tr.marginal) opt.mode = 2;
    opt.prior_kind = tr.prior_kind;
    opt.prior_mu = tr.prior_mu;
    opt.gl = c.gl;
    opt.pc = 0;
    opt.L_last = NAN;
    opt.last.ex = 0; opt.last.lm = 0.f;
    opt.last.g[0] = opt.last.g[1] = opt.last.h[0] = opt.last.h[1] = opt.last.h[2] = 0.f;
  }
  EvalOut res;
  for (int ev = 0; ev < kMaxTrialEvals; ev++) {
    if (tid == 0) {
      const bool more = !failed && opt.next(ev == 0 ? nullptr : &res);
      sm.ctrl->cmd = more ? (opt.req_derivs ? 2 : 1) : 0;
      sm.ctrl->pend = opt.req_p;
      sm.ctrl->dist = opt.req_d;
      sm.ctrl->prox = opt.req_x;
    }
    __syncthreads();
    const Ctrl ctl = *sm.ctrl;
    if (ctl.cmd == 0) break;
    const bool derivs = ctl.cmd == 2;
    {
      TrialSmem ts{};
      ts.E = sm.E; ts.Em1 = sm.Em1; ts.Lr = sm.Lr;
      trial_exps(ts, NM, K, ctl, tid, kTcThreads);
    }
    tc_scales(sm, NM, ctl, tid);
    __syncthreads();
    TcRows rw;
    if (nch > 0) tc_load_rows(c, sm, node, Sq, 0, 0, tid, rw);
    if (nch > 0 && !(derivs ? tc_query_tables<true>(c, sm, tmem, NM, ncz, nc, zc, tid, phase)
                            : tc_query_tables<false>(c, sm, tmem, NM, ncz, nc, zc, tid, phase)))
      failed = true;
    for (int r = 0; r < c.RP && nch > 0 && !failed; r++) {
      if (derivs) tc_btiles<true>(sm, NM, r, tid);
      else tc_btiles<false>(sm, NM, r, tid);
      // (the barrier at the top of the first chunk publishes the tables)
      for (int ch = 0; ch < nch; ch++) {
        const bool ok = derivs ? tc_chunk<true>(c, sm, tmem, node, Sq, r, ch, nch, cap, tid, phase, rw)
                               : tc_chunk<false>(c, sm, tmem, node, Sq, r, ch, nch, cap, tid, phase, rw);
        if (!ok) { failed = true; break; }
      }
    }
    if (failed) break;  // uniform: the completion check is a CTA-wide vote (recorded there)
    // ---- per-site products over the thread's sites, CTA reduction ----
    SiteAcc acc;
    acc.init();
    for (int i = tid; i < Sq; i += kTcThreads) {
      const float *a = sm.acc + i;
      if (derivs) acc.add(a[0], a[cap], a[2 * cap], a[3 * cap], a[4 * cap], a[5 * cap], true);
      else acc.add(a[0], 0.f, 0.f, 0.f, 0.f, 0.f, false);
    }
    for (int o = 16; o > 0; o >>= 1) {
      float mo = __shfl_down_sync(0xffffffffu, acc.m, o);
      int eo = __shfl_down_sync(0xffffffffu, acc.e, o);
      acc.m *= mo;
      acc.e += eo;
      int em;
      acc.m = frexpf(acc.m, &em);
      acc.e += em;
    }
    if (derivs) {
      acc.gp = warp_sum_f(acc.gp); acc.gd = warp_sum_f(acc.gd);
      acc.hpp = warp_sum_f(acc.hpp); acc.hdd = warp_sum_f(acc.hdd); acc.hpd = warp_sum_f(acc.hpd);
    }
    if (lane == 0) {
      sm.red[warp * 8 + 0] = acc.m;
      sm.redi[warp] = acc.e;
      sm.red[warp * 8 + 1] = acc.gp; sm.red[warp * 8 + 2] = acc.gd;
      sm.red[warp * 8 + 3] = acc.hpp; sm.red[warp * 8 + 4] = acc.hdd; sm.red[warp * 8 + 5] = acc.hpd;
    }
    __syncthreads();
    if (tid == 0) {
      float mt = 1.f, sg[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      int et = 0;
      for (int k = 0; k < kTcThreads / 32; k++) {
        mt *= sm.red[k * 8];
        et += sm.redi[k];
        int em;
        mt = frexpf(mt, &em);
        et += em;
        for (int j = 0; j < 5; j++) sg[j] += sm.red[k * 8 + 1 + j];
      }
      res.ex = et;
      res.lm = logf(mt);
      res.g[0] = sg[0]; res.g[1] = sg[1];
      res.h[0] = sg[2]; res.h[1] = sg[3]; res.h[2] = sg[4];
    }
  }
  if (tid == 0) {
    TrialRes rr;
    rr.like = failed ? NAN : opt.L_last;
    rr.pend = opt.pend;
    rr.dist = opt.dist;
    rr.der[0] = opt.last.g[0]; rr.der[1] = opt.last.g[1];
    rr.der[2] = opt.last.h[0]; rr.der[3] = opt.last.h[1]; rr.der[4] = opt.last.h[2];
    rr.der[5] = 0;
    rr.status = failed ? 1 : opt.status;
    rr.last = opt.last;
    rr.n_evals = opt.n_evals;
    *sm.res = rr;
    if (c.stats) {
      atomicAdd(&c.stats[0], (unsigned long long)opt.n_evals);
      atomicAdd(&c.stats[1], (unsigned long long)opt.n_evals * (unsigned long long)Sq);
    }
  }
  __syncthreads();
  return *sm.res;
}

// A batch of independent trials, one CTA each.
__global__ void __launch_bounds__(kTcThreads, 1) k_trials_tc(TrialCtx c, const TrialIn *__restrict__ trials,
                                                             const int *__restrict__ order, int n, TrialRes *out) {
  extern __shared__ __align__(16) char t_smem[];
  if (blockIdx.x >= n) return;
  const int tid = threadIdx.x;
  const int ti = order ? order[blockIdx.x] : blockIdx.x;
  const TcSmem sm = tc_carve(t_smem, c.cap, c.NM, c.ncode, c.zcodes);
  const uint32_t tmem = tc_setup(c, sm, tid);
  uint32_t phase = 0;
  bool failed = false;
  const TrialRes rr = tc_trial(c, sm, tmem, phase, failed, trials[ti], tid);
  if (tid == 0) out[ti] = rr;
  tc_teardown(sm, tmem, phase, failed, tid);
}
