// Stage-2 trials of 20-state Gamma-mixture models on the tensor cores: one
// team of 128 threads per (query, location) optimisation
// (Three_tax.optimize, pplacer_src/three_tax.ml:48-83), the per-site evolves
// of the distal and proximal GLVs (Gmix_model.evolve_into,
// gmix_model.ml:308-315) as tcgen05 MMAs.  Included by engine.cu inside its
// anonymous namespace, after trials.cuh.
//
// The operands are the GLVs in the eigenbasis of the rate matrix: with
// P(t) = X diag(exp(r lambda t)) X^-1, the evolved distal vector is
// X (e o X^-1 D), e = exp(r lambda t), and its t-derivatives put r lambda
// (or its square) beside e.  So the B operand of rate r -- the rows
// X[i][k] (r lambda_k)^m, m = 0, 1, 2 -- is a constant of the model: it is
// built once per CTA, in shared memory, and shared by the CTA's teams.  The
// A operand is the chunk's rows X^-1 D (darr_e / parr_e, built once per tree)
// times e at the evaluation's distal (proximal) length, written by each
// thread -- one per site, TMEM lane = site -- straight into tensor memory,
// split into TF32 hi / lo.
//
// A CTA holds one or two teams (as its shared memory allows); each team has
// its own named barrier, mbarrier and 256 TMEM columns: A operands at
// [0, 96) (distal hi, lo, proximal hi, lo; 24 columns each) and the
// accumulators at [128, 192) (distal) and [192, 256) (proximal).
//
// One evaluation at (pend, dist), per team:
//   thread 0: optimiser -> next point                      | barrier
//   all: exp factors of the three lengths                  | barrier
//   query tables: the statd-weighted evolved query vectors of every
//        character code (and d/dpend, d2/dpend2) for every rate, one MMA group
//        per 128 rows (X rows scaled by the pendant factors) x Lt (the codes'
//        vectors in the eigenbasis, a shared constant)     | barrier
//   per rate r, per chunk of 128 sites:
//     all: the chunk's rows (loaded during the previous MMAs) times the exp
//          factors, TF32 hi / lo into the team's A columns    | barrier
//     thread 0: 2 x 9 MMAs (3 K steps x 3 products) into the distal and
//               proximal accumulators; commit
//     all: load the next chunk's rows; wait for the MMAs; each thread reads
//          its site's TMEM lane and adds the rate's site likelihood (and
//          derivatives) into the site's accumulators (its own sites only)
//   all: per-site (mantissa, exponent) products and derivative sums, team
//        reduction                                                  | barrier
// Value-only evaluations use N = 32 (the P rows only).  Every wait on the
// MMA completion is bounded; on a timeout the kernel records the error, stops
// issuing, waits once more (bounded) and frees its TMEM.

constexpr int kTcThreads = pgb::tc::kTeamThreads;  // one team: thread t = TMEM lane t = site t of a chunk
constexpr int kTcMaxTeams = 2;                      // 2 x 256 TMEM columns fill the SM's 512
constexpr int kTcK = 20;
constexpr int kTcNDer = 64;     // B rows with derivatives: P, dP, d2P (3 x 20) + 4 zero rows
constexpr int kTcNVal = 32;     // B rows of a value-only evaluation: P (20) + 12 rows not read
constexpr int kTcCodeRows = 32; // rows of the codes' tile (N of the query-table MMA)
constexpr uint32_t kTcTeamCols = 256;                             // TMEM columns per team
constexpr uint32_t kTcAdH = 0, kTcAdL = 24, kTcAxH = 48, kTcAxL = 72;  // A: distal hi / lo, proximal hi / lo
constexpr uint32_t kTcDd = 128, kTcDx = 192;                         // accumulators: distal, proximal
constexpr int kTcBTile = kTcNDer * pgb::tc::kKPad;                   // floats of one B tile
constexpr int kTcLTile = kTcCodeRows * pgb::tc::kKPad;
constexpr int kTcXs = kTcK + 1;  // padded row stride of X (bank spread)
constexpr int kTcZs = kTcK + 1;  // padded row stride of the query-vector tables
constexpr int kTcMaxRates = 4;   // query-table rows 3 x 4 x 20 fit two 128-row MMA tiles
static_assert(pgb::kMaxCodes <= kTcCodeRows, "the query-vector table GEMM has N = 32 codes");

// One team's view of the CTA's shared memory.
struct TcSmem {
  // shared by the CTA's teams, written once by tc_setup
  float *bt;                          // [NM][2][kTcBTile] B tiles of each rate, TF32 hi / lo
  float *lt;                          // [2][kTcLTile] the codes' vectors in the eigenbasis, hi / lo
  float *X;                           // [K][kTcXs]
  float *Lr, *lv, *statd;             // [NM][K] rate * lambda, [ncode][K], [K]
  uint32_t *tbase;                    // the CTA's TMEM base
  // the team's own
  float *acc;                         // [6][cap] per-site sums over rates
  float *Z;                           // [3][NM][zcodes][kTcZs]: query vectors and d/dpend, d2/dpend2
  float *E, *Em1;                     // [3][NM][K]: exp / expm1 (r lambda t), t = dist, cut - dist, pend
  float *red;                         // [4][8]
  int *redi;                          // [4]
  uint16_t *col;                      // [cap] alignment columns of the query's sites
  uint8_t *code;                      // [cap]
  Ctrl *ctrl;
  Optimiser *opt;
  TrialRes *res;  // a finished trial's result, read by every thread of the team
  uint64_t *bar;
  int bar_id;     // the team's named barrier (1 + team)
};

__host__ __device__ inline size_t tc_shared_bytes(int NM, int ncode) {
  const int K = kTcK;
  size_t b = align16((size_t)NM * 2 * kTcBTile * 4) + align16((size_t)2 * kTcLTile * 4);
  b += align16((size_t)K * kTcXs * 4) + align16((size_t)NM * K * 4) + align16((size_t)ncode * K * 4);
  b += align16((size_t)K * 4) + 16;
  return b;
}
__host__ __device__ inline size_t tc_team_bytes(int cap, int NM, int zcodes) {
  const int K = kTcK;
  size_t b = align16((size_t)6 * cap * 4);
  b += align16((size_t)3 * NM * zcodes * kTcZs * 4);
  b += 2 * align16((size_t)3 * NM * K * 4);
  b += align16(4 * 8 * 4) + align16(4 * 4);
  b += align16((size_t)cap * 2) + align16((size_t)cap);
  b += align16(sizeof(Ctrl)) + align16(sizeof(Optimiser)) + align16(sizeof(TrialRes)) + 16;
  return b;
}
// zcodes: the character codes the query tables hold (the primary states,
// or every code when a query has ambiguity characters)
__host__ __device__ inline size_t tc_trial_smem_bytes(int cap, int NM, int ncode, int zcodes, int teams) {
  return tc_shared_bytes(NM, ncode) + (size_t)teams * tc_team_bytes(cap, NM, zcodes) + 128;  // + base alignment
}

__device__ inline TcSmem tc_carve(char *base, int cap, int NM, int ncode, int zcodes, int team) {
  const int K = kTcK;
  TcSmem s;
  char *p = (char *)(((uintptr_t)base + 127) & ~(uintptr_t)127);
  auto take = [&](size_t bytes) { char *r = p; p += align16(bytes); return r; };
  s.bt = (float *)take((size_t)NM * 2 * kTcBTile * 4);
  s.lt = (float *)take((size_t)2 * kTcLTile * 4);
  s.X = (float *)take((size_t)K * kTcXs * 4);
  s.Lr = (float *)take((size_t)NM * K * 4);
  s.lv = (float *)take((size_t)ncode * K * 4);
  s.statd = (float *)take((size_t)K * 4);
  s.tbase = (uint32_t *)take(16);
  p += (size_t)team * tc_team_bytes(cap, NM, zcodes);
  s.acc = (float *)take((size_t)6 * cap * 4);
  s.Z = (float *)take((size_t)3 * NM * zcodes * kTcZs * 4);
  s.E = (float *)take((size_t)3 * NM * K * 4);
  s.Em1 = (float *)take((size_t)3 * NM * K * 4);
  s.red = (float *)take(4 * 8 * 4);
  s.redi = (int *)take(4 * 4);
  s.col = (uint16_t *)take((size_t)cap * 2);
  s.code = (uint8_t *)take((size_t)cap);
  s.ctrl = (Ctrl *)take(sizeof(Ctrl));
  s.opt = (Optimiser *)take(sizeof(Optimiser));
  s.res = (TrialRes *)take(sizeof(TrialRes));
  s.bar = (uint64_t *)take(16);
  s.bar_id = 1 + team;
  return s;
}

// TMEM address of the thread's lane (t = team thread) at the team's base
__device__ __forceinline__ uint32_t tc_lane_addr(uint32_t tmem, int t) {
  return tmem + ((uint32_t)(32 * (t >> 5)) << 16);
}

// Records where a completion wait gave up (the first one in the launch).
__device__ __forceinline__ void tc_record_timeout(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, uint32_t phase,
                                                  bool mine, int r, int ch, int Sq, int nch) {
  namespace T = pgb::tc;
  if (c.tc_err && atomicCAS(c.tc_err, 0, 1) == 0) {
    int *d = c.tc_err;
    d[1] = blockIdx.x * kTcMaxTeams + (sm.bar_id - 1); d[2] = r; d[3] = ch; d[4] = (int)phase; d[5] = mine;
    d[6] = T::bar_test(sm.bar, phase); d[7] = T::bar_test(sm.bar, phase ^ 1u);
    d[8] = (int)tmem; d[9] = (int)T::smem_addr(sm.bt); d[10] = (int)T::smem_addr(sm.bar);
    d[11] = Sq; d[12] = nch;
    __threadfence();
  }
}

// Query tables of every rate on the tensor cores: rows rho = (m * NM + r) *
// 20 + i (m = 0: value, 1, 2: d/dpend, d2/dpend2) of A = X[i][.] * f(.), f
// = expm1(r lambda pend), r lambda e, (r lambda)^2 e; times Lt^T (the codes'
// likelihood vectors in the eigenbasis) gives sum_k X[i][k] f_k Lt[code][k],
// so that Z = statd_i * (lv[code][i] + that) for m = 0 (P = I + X diag(expm1)
// X^-1) and statd_i * that for the derivatives.  Rows 0..127 go through the
// distal A columns into accumulator columns [128, 160), rows 128.. through
// the proximal A columns into [160, 192).  Returns false when the
// completion wait timed out.
template <bool DER>
__device__ __forceinline__ bool tc_query_tables(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, int NM, int ncz,
                                                int zc, int t, uint32_t &phase) {
  namespace T = pgb::tc;
  const int K = kTcK;
  const int rows = (DER ? 3 : 1) * NM * K;  // <= 240
  const uint32_t tl = tc_lane_addr(tmem, t);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    if (h == 1 && rows <= T::kTileRows) break;  // uniform
    const int rho = t + h * T::kTileRows;
    float v[T::kKPad];
#pragma unroll
    for (int k = 0; k < T::kKPad; k++) v[k] = 0.f;
    if (rho < rows) {
      const int m = rho / (NM * K), r = (rho / K) % NM, i = rho % K;
      const float *x = sm.X + i * kTcXs, *lr = sm.Lr + r * K;
      const float *em = sm.Em1 + (2 * NM + r) * K, *e = sm.E + (2 * NM + r) * K;
#pragma unroll
      for (int k = 0; k < K; k++) v[k] = x[k] * (m == 0 ? em[k] : (m == 1 ? lr[k] : lr[k] * lr[k]) * e[k]);
    }
    T::st_split_row(tl, h == 0 ? kTcAdH : kTcAxH, h == 0 ? kTcAdL : kTcAxL, v);
  }
  T::st_wait();
  T::fence_before();
  T::team_sync(sm.bar_id);
  if (t == 0) {
    T::fence_after();
    const uint32_t id = T::idesc_tf32(T::kTileRows, 32);
    const uint32_t lh = T::smem_addr(sm.lt), ll = T::smem_addr(sm.lt + kTcLTile);
    T::mma_3xtf32_ts(tmem + kTcDd, tmem + kTcAdH, tmem + kTcAdL, lh, ll, id);
    if (rows > T::kTileRows) T::mma_3xtf32_ts(tmem + kTcDd + 32, tmem + kTcAxH, tmem + kTcAxL, lh, ll, id);
    T::commit(sm.bar);
  }
  const bool mine = T::bar_wait(sm.bar, phase);
  const bool ok = T::team_and(sm.bar_id, mine);
  if (!ok && t == 0) tc_record_timeout(c, sm, tmem, phase, mine, -1, -1, 0, 0);
  phase ^= 1u;
  T::fence_after();
  if (!ok) return false;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int rho = t + h * T::kTileRows;
    if (h == 1 && rows <= T::kTileRows) break;  // uniform
    float zv[32];
    {
      float t16[16];
      T::ld16(tl + kTcDd + 32 * h, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) zv[j] = t16[j];
      T::ld16(tl + kTcDd + 32 * h + 16, t16);
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

// One rate of one chunk: the A operands into TMEM, MMAs, then the epilogue
// adds the rate's site likelihood and derivatives into the site's
// accumulators.  Returns false when the completion wait timed out.
template <bool DER>
__device__ __forceinline__ bool tc_chunk(const TrialCtx &c, const TcSmem &sm, uint32_t tmem, int node, int Sq,
                                         int r, int ch, int nch, int cap, int t, uint32_t &phase, TcRows &rw) {
  namespace T = pgb::tc;
  const int K = kTcK, NM = c.NM;
  const uint32_t tl = tc_lane_addr(tmem, t);
  {
    // A rows: the eigen-coordinates times exp(r lambda t) at the distal and
    // proximal lengths (the previous MMAs, which read these columns, are done)
    const float *ed = sm.E + r * K, *ex = sm.E + (NM + r) * K;
    float v[T::kKPad];
#pragma unroll
    for (int k = K; k < T::kKPad; k++) v[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      v[4 * k] = ed[4 * k] * rw.d[k].x; v[4 * k + 1] = ed[4 * k + 1] * rw.d[k].y;
      v[4 * k + 2] = ed[4 * k + 2] * rw.d[k].z; v[4 * k + 3] = ed[4 * k + 3] * rw.d[k].w;
    }
    T::st_split_row(tl, kTcAdH, kTcAdL, v);
#pragma unroll
    for (int k = 0; k < 5; k++) {
      v[4 * k] = ex[4 * k] * rw.x[k].x; v[4 * k + 1] = ex[4 * k + 1] * rw.x[k].y;
      v[4 * k + 2] = ex[4 * k + 2] * rw.x[k].z; v[4 * k + 3] = ex[4 * k + 3] * rw.x[k].w;
    }
    T::st_split_row(tl, kTcAxH, kTcAxL, v);
  }
  T::st_wait();
  T::fence_before();
  T::team_sync(sm.bar_id);  // A rows written; the previous epilogue's TMEM reads done; Z published
  if (t == 0) {
    T::fence_after();
    const uint32_t id = T::idesc_tf32(T::kTileRows, DER ? kTcNDer : kTcNVal);
    const uint32_t bh = T::smem_addr(sm.bt + (size_t)r * 2 * kTcBTile), bl = bh + kTcBTile * 4;
    T::mma_3xtf32_ts(tmem + kTcDd, tmem + kTcAdH, tmem + kTcAdL, bh, bl, id);
    T::mma_3xtf32_ts(tmem + kTcDx, tmem + kTcAxH, tmem + kTcAxL, bh, bl, id);
    T::commit(sm.bar);
  }
  // the next chunk's rows (next rate's first chunk after the last) in flight
  // during the MMAs
  {
    int nr = r, nc2 = ch + 1;
    if (nc2 == nch) { nr = r + 1; nc2 = 0; }
    if (nr < c.RP) tc_load_rows(c, sm, node, Sq, nr, nc2, t, rw);
  }
  const bool mine = T::bar_wait(sm.bar, phase);
  const bool ok = T::team_and(sm.bar_id, mine);  // uniform over the team
  if (!ok && t == 0) tc_record_timeout(c, sm, tmem, phase, mine, r, ch, Sq, nch);
  phase ^= 1u;
  T::fence_after();
  if (!ok) return false;
  const int i = ch * T::kTileRows + t;
  const int code = i < Sq ? sm.code[i] : 0;
  const int zc = c.zcodes;
  const float *z = sm.Z + ((size_t)r * zc + code) * kTcZs;
  float u = 0.f, ud = 0.f, udd = 0.f, up = 0.f, upp = 0.f, upd = 0.f;
  if (DER) {
    float dv[64], xv[64];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      float t16[16];
      T::ld16(tl + kTcDd + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) dv[16 * b + j] = t16[j];
      T::ld16(tl + kTcDx + 16 * b, t16);
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
      T::ld16(tl + kTcDd + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) dv[16 * b + j] = t16[j];
      T::ld16(tl + kTcDx + 16 * b, t16);
#pragma unroll
      for (int j = 0; j < 16; j++) xv[16 * b + j] = t16[j];
    }
    T::ld_wait();
    T::pin(dv);
    T::pin(xv);
#pragma unroll
    for (int ii = 0; ii < K; ii++) u = fmaf(z[ii], dv[ii] * xv[ii], u);
  }
  if (i < Sq) {  // site i belongs to this thread in every rate
    float *a = sm.acc + i;
    if (r == 0) {
      a[0] = u;
      if (DER) { a[cap] = ud; a[2 * cap] = udd; a[3 * cap] = up; a[4 * cap] = upp; a[5 * cap] = upd; }
    } else {
      a[0] += u;
      if (DER) { a[cap] += ud; a[2 * cap] += udd; a[3 * cap] += up; a[4 * cap] += upp; a[5 * cap] += upd; }
    }
  }
  T::fence_before();  // the next chunk's barrier orders these TMEM reads before its MMAs
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

// Per-CTA setup of the tensor-core trial kernels, by every thread of the
// CTA (tid < nthreads): the shared model constants, the B tiles of every
// rate (rows m * 20 + i: X[i][k] (r lambda_k)^m, zero past the states and
// rows 60..63) and the codes' tile, TF32 hi / lo; teams x 256 TMEM columns;
// each team's mbarrier.  Returns the CTA's TMEM base.
__device__ __forceinline__ uint32_t tc_setup(const TrialCtx &c, const TcSmem &sm, int tid, int nthreads, int teams) {
  namespace T = pgb::tc;
  const int K = kTcK, NM = c.NM, nc = c.ncode;
  for (int it = tid; it < K * K; it += nthreads) {
    const int i = it / K, k = it - i * K;
    sm.X[i * kTcXs + k] = c.X[it];
  }
  for (int it = tid; it < nc * K; it += nthreads) sm.lv[it] = c.lvf[it];
  for (int it = tid; it < NM * K; it += nthreads) sm.Lr[it] = c.rates[it / K] * c.lam[it % K];
  if (tid < K) sm.statd[tid] = c.statd[tid];
  for (int it = tid; it < NM * kTcNDer * T::kKPad; it += nthreads) {
    const int r = it / (kTcNDer * T::kKPad), rem = it - r * kTcNDer * T::kKPad;
    const int n = rem / T::kKPad, k = rem - n * T::kKPad;
    float v = 0.f;
    if (n < 3 * K && k < K) {
      const int m = n / K, i = n - m * K;
      const float lr = c.rates[r] * c.lam[k];
      v = c.X[i * K + k] * (m == 0 ? 1.f : (m == 1 ? lr : lr * lr));
    }
    float hi, lo;
    T::split_tf32(v, hi, lo);
    float *b = sm.bt + (size_t)r * 2 * kTcBTile;
    b[T::off(n, k)] = hi;
    b[kTcBTile + T::off(n, k)] = lo;
  }
  for (int it = tid; it < kTcLTile; it += nthreads) {
    const int n = it / T::kKPad, k = it - n * T::kKPad;
    const float v = (n < nc && k < K) ? c.Lt[n * K + k] : 0.f;
    float hi, lo;
    T::split_tf32(v, hi, lo);
    sm.lt[T::off(n, k)] = hi;
    sm.lt[kTcLTile + T::off(n, k)] = lo;
  }
  T::fence_async_smem();  // the tiles become visible to the tensor core
  if ((tid & (kTcThreads - 1)) == 0) T::bar_init(sm.bar, 1);  // each team's thread 0: its own mbarrier
  __syncwarp();
  if ((tid >> 5) == 0) T::tmem_alloc(sm.tbase, kTcTeamCols * (uint32_t)teams);
  T::fence_before();
  __syncthreads();
  T::fence_after();
  return *sm.tbase;
}

// After the team's last trial: a timed-out MMA group is waited for once more
// (bounded).  Then, with every team done, the TMEM columns are freed.
__device__ __forceinline__ void tc_teardown(const TcSmem &sm, uint32_t phase, bool failed, int tid, int teams) {
  namespace T = pgb::tc;
  if (failed) T::bar_wait(sm.bar, phase ^ 1u);
  T::fence_before();
  __syncthreads();
  T::fence_after();
  if ((tid >> 5) == 0) T::tmem_dealloc(*sm.tbase, kTcTeamCols * (uint32_t)teams);
}

// One trial (Three_tax.optimize at one location, or its marginal
// likelihood) by a team; every thread of the team returns the same result
// (tid: the thread's index in the team).  failed is
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
  T::team_sync(sm.bar_id);  // the previous trial's readers of red / res are done
  if (lane == 0) reinterpret_cast<long long *>(sm.red)[warp] = esum;
  T::team_sync(sm.bar_id);
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
    opt.pp_rule = c.pp_rule;
    opt.pp_rel = c.pp_rel_err;
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
    T::team_sync(sm.bar_id);
    const Ctrl ctl = *sm.ctrl;
    if (ctl.cmd == 0) break;
    const bool derivs = ctl.cmd == 2;
    {
      TrialSmem ts{};
      ts.E = sm.E; ts.Em1 = sm.Em1; ts.Lr = sm.Lr;
      trial_exps(ts, NM, K, ctl, tid, kTcThreads);
    }
    T::team_sync(sm.bar_id);
    TcRows rw;
    if (nch > 0) tc_load_rows(c, sm, node, Sq, 0, 0, tid, rw);
    if (nch > 0 && !(derivs ? tc_query_tables<true>(c, sm, tmem, NM, ncz, zc, tid, phase)
                            : tc_query_tables<false>(c, sm, tmem, NM, ncz, zc, tid, phase)))
      failed = true;
    for (int r = 0; r < c.RP && nch > 0 && !failed; r++) {
      // (the barrier before the first chunk's MMAs publishes the tables)
      for (int ch = 0; ch < nch; ch++) {
        const bool ok = derivs ? tc_chunk<true>(c, sm, tmem, node, Sq, r, ch, nch, cap, tid, phase, rw)
                               : tc_chunk<false>(c, sm, tmem, node, Sq, r, ch, nch, cap, tid, phase, rw);
        if (!ok) { failed = true; break; }
      }
    }
    if (failed) break;  // uniform: the completion check is a team-wide vote (recorded there)
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
    T::team_sync(sm.bar_id);
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
  T::team_sync(sm.bar_id);
  return *sm.res;
}

// A batch of independent trials, one CTA (one team) each.
__global__ void __launch_bounds__(kTcThreads, 1) k_trials_tc(TrialCtx c, const TrialIn *__restrict__ trials,
                                                             const int *__restrict__ order, int n, TrialRes *out) {
  extern __shared__ __align__(16) char t_smem[];
  if (blockIdx.x >= n) return;
  const int tid = threadIdx.x;
  const int ti = order ? order[blockIdx.x] : blockIdx.x;
  const TcSmem sm = tc_carve(t_smem, c.cap, c.NM, c.ncode, c.zcodes, 0);
  const uint32_t tmem = tc_setup(c, sm, tid, kTcThreads, 1);
  uint32_t phase = 0;
  bool failed = false;
  const TrialRes rr = tc_trial(c, sm, tmem, phase, failed, trials[ti], tid);
  if (tid == 0) out[ti] = rr;
  tc_teardown(sm, phase, failed, tid, 1);
}
