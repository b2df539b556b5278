// Stage-2 trials of 20-state Gamma-mixture models on the tensor cores: one
// CTA of 128 threads per (query, location) optimisation (Three_tax.optimize,
// pplacer_src/three_tax.ml:285-320), the per-site evolves of the distal and
// proximal GLVs (Gmix_model.evolve_into, gmix_model.ml:308-315) as tcgen05
// MMAs.  Included by engine.cu inside its anonymous namespace, after
// trials.cuh.
//
// One evaluation at (pend, dist):
//   thread 0: optimiser -> next point                      | barrier
//   all: exp factors of the three lengths                  | barrier
//   per rate r:
//     all: B tiles of rate r -- the rows of P, dP, d2P at dist (distal) and
//          at cut - dist (proximal), TF32 hi / lo -- and the statd-weighted
//          query vectors per character (and d/dpend, d2/dpend2)   | barrier
//     per chunk of 128 sites:
//       all: the chunk's darr / parr rows (loaded during the previous
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

struct TcSmem {
  float *a_dh, *a_dl, *a_xh, *a_xl;  // A tiles [128 x 24]: distal / proximal rows, hi / lo
  float *b_dh, *b_dl, *b_xh, *b_xl;  // B tiles [64 x 24]
  float *acc;                         // [6][cap] per-site sums over rates
  float *Z, *Z1, *Z2;                 // [ncode][kTcZs] of the current rate
  float *X, *Xit;                     // [K][kTcXs]
  float *E, *Em1, *Lr;                // [3][NM][K], [3][NM][K], [NM][K]
  float *Lt, *lv, *statd;
  float *red;                         // [4][8]
  int *redi;                          // [4]
  uint16_t *col;                      // [cap] alignment columns of the query's sites
  uint8_t *code;                      // [cap]
  Ctrl *ctrl;
  Optimiser *opt;
  uint64_t *bar;
  uint32_t *tbase;
};

__host__ __device__ inline size_t tc_trial_smem_bytes(int cap, int NM, int ncode) {
  const int K = kTcK;
  size_t b = 4 * align16((size_t)pgb::tc::kTileFloats * 4) + 4 * align16((size_t)kTcNDer * pgb::tc::kKPad * 4);
  b += align16((size_t)6 * cap * 4);
  b += 3 * align16((size_t)ncode * kTcZs * 4);
  b += 2 * align16((size_t)K * kTcXs * 4);
  b += 2 * align16((size_t)3 * NM * K * 4) + align16((size_t)NM * K * 4);
  b += 2 * align16((size_t)ncode * K * 4) + align16((size_t)K * 4);
  b += align16(4 * 8 * 4) + align16(4 * 4);
  b += align16((size_t)cap * 2) + align16((size_t)cap);
  b += align16(sizeof(Ctrl)) + align16(sizeof(Optimiser)) + 16 + 16;
  return b + 1024;  // base alignment of the operand tiles
}

__device__ inline TcSmem tc_carve(char *base, int cap, int NM, int ncode) {
  const int K = kTcK;
  TcSmem s;
  char *p = (char *)(((uintptr_t)base + 1023) & ~(uintptr_t)1023);
  auto take = [&](size_t bytes) { char *r = p; p += align16(bytes); return r; };
  const size_t at = (size_t)pgb::tc::kTileFloats * 4, bt = (size_t)kTcNDer * pgb::tc::kKPad * 4;
  s.a_dh = (float *)take(at); s.a_dl = (float *)take(at); s.a_xh = (float *)take(at); s.a_xl = (float *)take(at);
  s.b_dh = (float *)take(bt); s.b_dl = (float *)take(bt); s.b_xh = (float *)take(bt); s.b_xl = (float *)take(bt);
  s.acc = (float *)take((size_t)6 * cap * 4);
  const size_t zb = (size_t)ncode * kTcZs * 4;
  s.Z = (float *)take(zb); s.Z1 = (float *)take(zb); s.Z2 = (float *)take(zb);
  s.X = (float *)take((size_t)K * kTcXs * 4);
  s.Xit = (float *)take((size_t)K * kTcXs * 4);
  s.E = (float *)take((size_t)3 * NM * K * 4);
  s.Em1 = (float *)take((size_t)3 * NM * K * 4);
  s.Lr = (float *)take((size_t)NM * K * 4);
  s.Lt = (float *)take((size_t)ncode * K * 4);
  s.lv = (float *)take((size_t)ncode * K * 4);
  s.statd = (float *)take((size_t)K * 4);
  s.red = (float *)take(4 * 8 * 4);
  s.redi = (int *)take(4 * 4);
  s.col = (uint16_t *)take((size_t)cap * 2);
  s.code = (uint8_t *)take((size_t)cap);
  s.ctrl = (Ctrl *)take(sizeof(Ctrl));
  s.opt = (Optimiser *)take(sizeof(Optimiser));
  s.bar = (uint64_t *)take(16);
  s.tbase = (uint32_t *)take(16);
  return s;
}

// B tiles of rate r: row m * 20 + i, column j = (d^m/dt^m P(t))[i][j] at
// t = dist (distal tiles) and t = cut - dist (proximal tiles), from
// P = I + X diag(expm1(r lambda t)) X^-1 and its derivatives; plus the
// statd-weighted evolved query vectors of codes 0 .. ncz - 1 at pend.
template <bool DER>
__device__ __forceinline__ void tc_rate_tables(const TcSmem &sm, int NM, int r, int ncz, int tid) {
  const int K = kTcK;
  for (int it = tid; it < 2 * K * K; it += kTcThreads) {
    const int g = it / (K * K), ij = it - g * K * K;
    const int i = ij / K, j = ij - i * K;
    const float *xi = sm.X + i * kTcXs, *xj = sm.Xit + j * kTcXs;
    const float *em = sm.Em1 + (g * NM + r) * K;
    const float *e = sm.E + (g * NM + r) * K;
    const float *lr = sm.Lr + r * K;
    float a = i == j ? 1.f : 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll 5
    for (int k = 0; k < K; k++) {
      const float w = xi[k] * xj[k];
      a = fmaf(w, em[k], a);
      if (DER) {
        const float t1 = w * lr[k] * e[k];
        a1 += t1;
        a2 = fmaf(t1, lr[k], a2);
      }
    }
    float *bh = g == 0 ? sm.b_dh : sm.b_xh, *bl = g == 0 ? sm.b_dl : sm.b_xl;
    float h, l;
    pgb::tc::split_tf32(a, h, l);
    bh[pgb::tc::off(i, j)] = h;
    bl[pgb::tc::off(i, j)] = l;
    if (DER) {
      pgb::tc::split_tf32(a1, h, l);
      bh[pgb::tc::off(K + i, j)] = h;
      bl[pgb::tc::off(K + i, j)] = l;
      pgb::tc::split_tf32(a2, h, l);
      bh[pgb::tc::off(2 * K + i, j)] = h;
      bl[pgb::tc::off(2 * K + i, j)] = l;
    }
  }
  for (int it = tid; it < ncz * K; it += kTcThreads) {
    const int code = it / K, i = it - code * K;
    const float *x = sm.X + i * kTcXs;
    const float *lt = sm.Lt + code * K;
    const float *em = sm.Em1 + (2 * NM + r) * K;
    const float *e = sm.E + (2 * NM + r) * K;
    const float *lr = sm.Lr + r * K;
    float a = sm.lv[code * K + i], a1 = 0.f, a2 = 0.f;
#pragma unroll 5
    for (int k = 0; k < K; k++) {
      a = fmaf(x[k] * em[k], lt[k], a);
      if (DER) {
        const float t1 = x[k] * lr[k] * e[k] * lt[k];
        a1 += t1;
        a2 = fmaf(t1, lr[k], a2);
      }
    }
    const float pi = sm.statd[i];
    sm.Z[code * kTcZs + i] = pi * a;
    if (DER) {
      sm.Z1[code * kTcZs + i] = pi * a1;
      sm.Z2[code * kTcZs + i] = pi * a2;
    }
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
    const float4 *dp = reinterpret_cast<const float4 *>(c.darr + o);
    const float4 *xp = reinterpret_cast<const float4 *>(c.parr + o);
#pragma unroll
    for (int k = 0; k < 5; k++) { rw.d[k] = __ldg(dp + k); rw.x[k] = __ldg(xp + k); }
  } else {
#pragma unroll
    for (int k = 0; k < 5; k++) rw.d[k] = rw.x[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}
__device__ __forceinline__ void tc_store_split(float *hi, float *lo, int row, int k, float4 v) {
  float4 h, l;
  pgb::tc::split_tf32(v.x, h.x, l.x);
  pgb::tc::split_tf32(v.y, h.y, l.y);
  pgb::tc::split_tf32(v.z, h.z, l.z);
  pgb::tc::split_tf32(v.w, h.w, l.w);
  *reinterpret_cast<float4 *>(hi + pgb::tc::off(row, k)) = h;
  *reinterpret_cast<float4 *>(lo + pgb::tc::off(row, k)) = l;
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
  const float *z = sm.Z + code * kTcZs;
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
    const float *z1 = sm.Z1 + code * kTcZs, *z2 = sm.Z2 + code * kTcZs;
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

__global__ void __launch_bounds__(kTcThreads, 1) k_trials_tc(TrialCtx c, const TrialIn *__restrict__ trials,
                                                             const int *__restrict__ order, int n, TrialRes *out) {
  namespace T = pgb::tc;
  extern __shared__ __align__(16) char t_smem[];
  if (blockIdx.x >= n) return;
  const int K = kTcK;
  const int ti = order ? order[blockIdx.x] : blockIdx.x;
  const TrialIn tr = trials[ti];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NM = c.NM, nc = c.ncode, cap = c.cap;
  const TcSmem sm = tc_carve(t_smem, cap, NM, nc);
  const int q = tr.q, node = tr.node;
  const int Sq = c.qlen[q];
  const int ncz = c.qamb[q] > 0 ? nc : c.prim;
  const int nch = (Sq + T::kTileRows - 1) / T::kTileRows;
  // ---- prologue: model constants, the query's sites, TMEM, mbarrier ----
  for (int it = tid; it < K * K; it += kTcThreads) {
    const int i = it / K, k = it - i * K;
    sm.X[i * kTcXs + k] = c.X[it];
    sm.Xit[i * kTcXs + k] = c.Xit[it];
  }
  for (int it = tid; it < nc * K; it += kTcThreads) { sm.Lt[it] = c.Lt[it]; sm.lv[it] = c.lvf[it]; }
  for (int it = tid; it < NM * K; it += kTcThreads) sm.Lr[it] = c.rates[it / K] * c.lam[it % K];
  if (tid < K) sm.statd[tid] = c.statd[tid];
  // the padding columns 20..23 of every tile and the rows 60..63 of the B
  // tiles stay zero; the rest is rewritten before each use
  for (int it = tid; it < T::kTileFloats; it += kTcThreads) {
    sm.a_dh[it] = 0.f; sm.a_dl[it] = 0.f; sm.a_xh[it] = 0.f; sm.a_xl[it] = 0.f;
  }
  for (int it = tid; it < kTcNDer * T::kKPad; it += kTcThreads) {
    sm.b_dh[it] = 0.f; sm.b_dl[it] = 0.f; sm.b_xh[it] = 0.f; sm.b_xl[it] = 0.f;
  }
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
  if (lane == 0) reinterpret_cast<long long *>(sm.red)[warp] = esum;
  __syncwarp();
  if (warp == 0) T::tmem_alloc(sm.tbase, kTcCols);
  if (tid == 0) T::bar_init(sm.bar, 1);
  T::fence_before();
  __syncthreads();
  T::fence_after();
  const uint32_t tmem = *sm.tbase;
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
  uint32_t phase = 0;
  bool failed = false;
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
    __syncthreads();
    TcRows rw;
    if (nch > 0) tc_load_rows(c, sm, node, Sq, 0, 0, tid, rw);
    for (int r = 0; r < c.RP && !failed; r++) {
      if (derivs) tc_rate_tables<true>(sm, NM, r, ncz, tid);
      else tc_rate_tables<false>(sm, NM, r, ncz, tid);
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
  if (failed) T::bar_wait(sm.bar, phase ^ 1u);  // the timed-out MMAs, bounded, before the columns are freed
  T::fence_before();
  __syncthreads();
  if (warp == 0) T::tmem_dealloc(tmem, kTcCols);
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
    out[ti] = rr;
    if (c.stats) {
      atomicAdd(&c.stats[0], (unsigned long long)opt.n_evals);
      atomicAdd(&c.stats[1], (unsigned long long)opt.n_evals * (unsigned long long)Sq);
    }
  }
}
