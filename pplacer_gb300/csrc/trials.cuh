// Stage-2 trials: one CTA per (query, location) branch-length optimisation
// (Three_tax.optimize, pplacer_src/three_tax.ml:48-83, with the retry from
// default lengths of core.ml:272-279).  Included by engine.cu inside its
// anonymous namespace.
//
// Structure of the kernel: the query's informative sites of darr / parr[node]
// are gathered into shared memory once.  Warp 0 runs the optimiser as a state
// machine (a coroutine: each resume consumes one objective value and yields
// the next point); all warps then evaluate that point together.  One
// evaluation is three block barriers:
//   warp 0: decide next point, exp factors   | barrier A
//   all:    P(t) and derivative matrices,    | barrier B
//           evolved query vectors per character
//   all:    sites -> warp partials           | barrier C
//   warp 0: combine partials
// Every loop is bounded and every path through warp 0 ends with the stop
// command, so the barriers always complete.

constexpr int kTrialMaxWarps = 8;  // CTAs of 128 or 256 threads (autotuned per bin)
constexpr int kMaxTrialEvals = 200000;

// One evaluation: logL = ex * ln2 + lm + (trial constant); derivatives FP32.
struct EvalOut {
  int ex;
  float lm;
  float g[2], h[3];
};

struct TrialIn {
  int q, node;
  double pend0, dist0, tol;
  int seeded;    // the Newton form: seed is the evaluation at (pend0, dist0)
  EvalOut seed;  //   (derivatives included), which it then does not redo
  int marginal;     // 1: the marginal likelihood (mode 2) around (pend0, dist0)
  int prior_kind;   //   pendant prior: 0 uniform, 1 exponential
  double prior_mu;  //   mean of the exponential
};
struct TrialRes {
  double like, pend, dist;
  double der[6];
  int status, n_evals;
  EvalOut last;  // the evaluation at (pend, dist)
};

struct TrialCtx {
  const float *darr, *parr;
  const int *dexp, *pexp;
  int S, RP, K, NM, ncode, gcat;
  const double *bl;
  const uint16_t *reind;
  const uint8_t *mcode;
  const uint32_t *rcode;  // (category << 24) | (column << 8) | code; category 0 but for CAT
  const int *qamb;        // informative ambiguity characters per query
  int prim;               // primary (one-hot) character codes: 0 .. prim - 1
  const int *qlen;
  const uint8_t *site_cat;
  const float *X, *W, *Lt, *lvf, *statd, *lam, *rates;
  const float *Xit;           // X^-T (K x K): the tensor-core kernel's P(t) = I + X diag(.) Xit^T
  int *tc_err;                // [16]: [0] set when a tensor-core completion wait timed out, then where
  const float *darr_e, *parr_e;  // darr / parr rows times X^-1 (the tensor-core and eigen warp kernels' operands)
  int eig_ord;                // nucleotide eigen warp form: byte 0 the zero eigenvalue, bytes 1..3 the others
  int zcodes;                 // character codes of the tensor-core kernel's query tables
  double log_nrates;
  double start_pend, max_pend;
  int optimizer, mode;
  int smem_win, cap;
  unsigned long long *stats;  // [0] objective evaluations, [1] site evaluations
  const double *gl;           // Gauss-Legendre rule on [-1, 1]: kGlPoints nodes, then weights
  int pp_rule;                // marginal likelihood: 0 Gauss-Legendre panels, 1 the reference's nested QNG
  double pp_rel_err;          // the QNG's relative error (pp_rel_err, prefs.ml)
};

constexpr int kGlPoints = 12;  // nodes per panel of the marginal-likelihood quadrature

struct Ctrl {
  float pend, dist, prox;
  int cmd;  // 0 stop, 1 value, 2 value + derivatives
};


// logL difference a - b without FP64 (exact exponent difference)
__device__ __forceinline__ float dlogl(const EvalOut &a, const EvalOut &b) {
  return (float)(a.ex - b.ex) * 0.69314718f + (a.lm - b.lm);
}

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// shared memory of one trial CTA
struct TrialSmem {
  float *D, *P;              // [RP][cap][K] windows (smem_win)
  uint8_t *code, *cat;       // [cap]
  float *Md, *Mp, *Md1, *Md2, *Mp1, *Mp2;  // [NM][K][K]
  float *Z, *Z1, *Z2;        // [NM][ncode][K] statd-weighted evolved query vectors
  float *E, *Em1, *Lr;       // exp / expm1 factors [3][NM][K]; rate * lambda [NM][K]
  float *Tc;                 // the CAT eigenbasis form: per category [12] (exp factors, rate * lambda)
  float *X, *W, *Lt, *lv, *statd;  // model constants (W only for K = 4)
  float *red;                // [warps][8]
  int *redi;                 // [warps]
  Ctrl *ctrl;
  void *opt;  // the warp kernels' optimiser state (one per warp)
  TrialRes *res;  // the CTA form's finished trial, read by every thread
};

__host__ __device__ inline size_t trial_smem_bytes(int cap, int win, int RP, int K, int NM, int ncode) {
  size_t b = 0;
  if (win) b += 2 * align16((size_t)RP * cap * K * 4);
  b += 2 * align16((size_t)cap);
  b += 6 * align16((size_t)NM * K * K * 4);
  b += 3 * align16((size_t)NM * ncode * K * 4);
  b += 2 * align16((size_t)3 * NM * K * 4) + align16((size_t)NM * K * 4);
  b += align16((size_t)K * K * 4) + (K == 4 ? align16((size_t)K * K * K * 4) : 0) +
       2 * align16((size_t)ncode * K * 4) + align16((size_t)K * 4);
  b += align16(kTrialMaxWarps * 8 * 4) + align16(kTrialMaxWarps * 4);
  b += align16(sizeof(Ctrl)) + align16(sizeof(TrialRes));
  return b;
}

__device__ inline TrialSmem carve(char *base, int cap, int win, int RP, int K, int NM, int ncode) {
  TrialSmem s;
  char *p = base;
  auto take = [&](size_t bytes) { char *r = p; p += align16(bytes); return r; };
  s.D = win ? (float *)take((size_t)RP * cap * K * 4) : nullptr;
  s.P = win ? (float *)take((size_t)RP * cap * K * 4) : nullptr;
  s.code = (uint8_t *)take(cap);
  s.cat = (uint8_t *)take(cap);
  size_t mb = (size_t)NM * K * K * 4;
  s.Md = (float *)take(mb); s.Mp = (float *)take(mb); s.Md1 = (float *)take(mb);
  s.Md2 = (float *)take(mb); s.Mp1 = (float *)take(mb); s.Mp2 = (float *)take(mb);
  size_t zb = (size_t)NM * ncode * K * 4;
  s.Z = (float *)take(zb); s.Z1 = (float *)take(zb); s.Z2 = (float *)take(zb);
  s.E = (float *)take((size_t)3 * NM * K * 4);
  s.Em1 = (float *)take((size_t)3 * NM * K * 4);
  s.Lr = (float *)take((size_t)NM * K * 4);
  s.X = (float *)take((size_t)K * K * 4);
  s.W = K == 4 ? (float *)take((size_t)K * K * K * 4) : nullptr;
  s.Lt = (float *)take((size_t)ncode * K * 4);
  s.lv = (float *)take((size_t)ncode * K * 4);
  s.statd = (float *)take((size_t)K * 4);
  s.red = (float *)take(kTrialMaxWarps * 8 * 4);
  s.redi = (int *)take(kTrialMaxWarps * 4);
  s.ctrl = (Ctrl *)take(sizeof(Ctrl));
  s.res = (TrialRes *)take(sizeof(TrialRes));
  return s;
}

// ---------------------------------------------------------------------------
// Warp-0 optimiser state machines.  next(res) consumes the value of the last
// requested point (res == nullptr on the first call) and either sets the next
// request (req_*) and returns true, or finishes and returns false.
// ---------------------------------------------------------------------------
#define PGB_YIELD(label) \
  do {                   \
    pc = label;          \
    return true;         \
    case label:;         \
  } while (0)

// One QNG integral of the reference's posterior-probability integral
// (Gsl.Integration.qng, pplacer_src/integration.ml:27-31; QUADPACK's
// non-adaptive 21/43/87-point Gauss-Kronrod-Patterson scheme) fed one
// function value at a time, in the order QNG evaluates them: point j of
// [a, b] is node(j, a, b); accept(j, f) returns 0 for the next point, 1 when
// a stage met the tolerance (result), 2 when the 87-point stage failed
// (GSL_ETOL).  buf holds the 20 values of the 21-point stage, then the pair
// sums f(c + h x) + f(c - h x) the later stages reuse.
struct QngAcc {
  double fc, res10, res21, res43, res87, resabs, resasc, first, result;
  float buf[21];

  __device__ static double node(int j, double a, double b) {
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    if (j == 0) return c;
    double x;
    int i;
    if (j <= 10) { i = j - 1; x = pgb::qng::x1[i >> 1]; }
    else if (j <= 20) { i = j - 11; x = pgb::qng::x2[i >> 1]; }
    else if (j <= 42) { i = j - 21; x = pgb::qng::x3[i >> 1]; }
    else { i = j - 43; x = pgb::qng::x4[i >> 1]; }
    return (i & 1) ? c - h * x : c + h * x;
  }
  // rescale_error of QUADPACK: the stage difference scaled by the
  // integrand's variation, at least 50 eps |integral|
  __device__ static double rescale(double err, double rabs, double rasc) {
    err = fabs(err);
    if (rasc != 0.0 && err != 0.0) {
      const double scale = pow(200.0 * err / rasc, 1.5);
      err = scale < 1.0 ? rasc * scale : rasc;
    }
    if (rabs > 2.2250738585072014e-308 / (50.0 * 2.220446049250313e-16)) {
      const double min_err = 50.0 * 2.220446049250313e-16 * rabs;
      if (min_err > err) err = min_err;
    }
    return err;
  }
  __device__ int accept(int j, double f, double half, double epsrel) {
    namespace Q = pgb::qng;
    if (j == 0) { fc = f; return 0; }
    if (j <= 20) {
      buf[j - 1] = (float)f;
      if (j < 20) return 0;
      res10 = 0.0;
      res21 = Q::w21b[5] * fc;
      resabs = Q::w21b[5] * fabs(fc);
      for (int k = 0; k < 5; k++) {
        const double a1 = buf[2 * k], a2 = buf[2 * k + 1], s = a1 + a2;
        res10 += Q::w10[k] * s;
        res21 += Q::w21a[k] * s;
        resabs += Q::w21a[k] * (fabs(a1) + fabs(a2));
      }
      for (int k = 0; k < 5; k++) {
        const double a1 = buf[10 + 2 * k], a2 = buf[11 + 2 * k];
        res21 += Q::w21b[k] * (a1 + a2);
        resabs += Q::w21b[k] * (fabs(a1) + fabs(a2));
      }
      resabs *= fabs(half);
      const double mean = 0.5 * res21;
      resasc = Q::w21b[5] * fabs(fc - mean);
      for (int k = 0; k < 5; k++)
        resasc += Q::w21a[k] * (fabs(buf[2 * k] - mean) + fabs(buf[2 * k + 1] - mean)) +
                  Q::w21b[k] * (fabs(buf[10 + 2 * k] - mean) + fabs(buf[11 + 2 * k] - mean));
      resasc *= fabs(half);
      for (int k = 0; k < 10; k++) buf[k] = buf[2 * k] + buf[2 * k + 1];  // pair sums, in place
      result = res21 * half;
      if (rescale((res21 - res10) * half, resabs, resasc) < epsrel * fabs(result)) return 1;
      res43 = Q::w43b[11] * fc;
      for (int k = 0; k < 10; k++) res43 += buf[k] * Q::w43a[k];
      return 0;
    }
    if (j <= 42) {
      const int i = j - 21;
      if (!(i & 1)) { first = f; return 0; }
      const double s = first + f;
      res43 += s * Q::w43b[i >> 1];
      buf[10 + (i >> 1)] = (float)s;
      if (j < 42) return 0;
      result = res43 * half;
      if (rescale((res43 - res21) * half, resabs, resasc) < epsrel * fabs(result)) return 1;
      res87 = Q::w87b[22] * fc;
      for (int k = 0; k < 21; k++) res87 += buf[k] * Q::w87a[k];
      return 0;
    }
    const int i = j - 43;
    if (!(i & 1)) { first = f; return 0; }
    res87 += Q::w87b[i >> 1] * (first + f);
    if (j < 86) return 0;
    result = res87 * half;
    return rescale((res87 - res43) * half, resabs, resasc) < epsrel * fabs(result) ? 1 : 2;
  }
};

struct Optimiser {
  // inputs
  int optimizer, mode;
  double cut, tol, max_pend, start_pend, pend0, dist0, cst;
  // outputs
  int status, n_evals;
  double pend, dist, prox;  // three-taxon state (three_tax.ml:15-21)
  double L_last;
  EvalOut last;
  // request
  float req_p, req_d, req_x;
  bool req_derivs;
  // coroutine
  int pc, qpc;  // next()'s and marg_qng()'s resume points
  int attempt;
  // Brent replica state
  int outer, which, iter, bstep, err;
  double prev_pend, prev_dist, cres[2];
  double raw, left, right, lefty, righty, smaller, miny, prevx, pv;
  double xl, xu, xm, fl, fu, fm, v, w, fv, fw, bd, be, u, fz, z, probe_dx, fval, fx;
  bool probe;
  // marginal likelihood state (mode 2)
  int prior_kind;
  double prior_mu;
  const double *gl;
  int pp_rule;    // 0: Gauss-Legendre panels; 1: the reference's nested QNG (to pp_rel)
  double pp_rel;
  double base, tgt, lo_b, hi_b, stp, sig_p, sig_d, qp, qd;
  int k_srch;
  union {
    struct {  // Gauss-Legendre panels
      double acc_in, acc_out, wd;
      double ppan[3], dpan[3];
      int n_ppan, n_dpan, ipan, jpan, ip, jd;
    };
    struct {  // nested QNG: inner (pendant) and outer (distal) integrals
      QngAcc qi, qo;
      double qU;
      int ij, oj, n_exc, qerr;
    };
  };
  // Newton state
  bool seeded;
  EvalOut seed;
  int it, ls, stall;
  float p, d, sp, sd, np, nd, allow, pred;
  bool accepted;
  EvalOut cur;

  __device__ double full(const EvalOut &o) const { return (double)o.ex * kLn2 + (double)o.lm + cst; }

  // Newton stops when the first-order gain g . s of its next (or last) step
  // is below this (logL units): 1e-2 in the stage-2 pass (pplacer's
  // tolerance 0.01, whose Brent stops within about 0.05 logL of the
  // optimum), 1e-7 in the final 1e-5 pass -- plus the evaluation's rounding
  // allowance.  A step-size rule alone is unsound here: near a zero pendant
  // the curvature is huge and Newton steps are tiny while the gradient is not.
  __device__ float newton_gain_tol() const { return tol >= 1e-3 ? 1e-2f : 1e-7f; }

  // log of the pendant prior density (core.ml:86-92): uniform 1 or
  // Gsl.Randist.exponential_pdf with mean mu
  __device__ double log_prior(double pnd) const { return prior_kind == 0 ? 0.0 : -log(prior_mu) - pnd / prior_mu; }
  __device__ double value_of(const EvalOut &o, double pnd) const { return full(o) + log_prior(pnd); }

  // find_upper_limit's objective at pendant x from the last evaluation:
  // |target - (L + log prior)|, an infinite value as 1e5 (three_tax.ml:142-148)
  __device__ double qng_objective(double x) const {
    const double y = fabs(tgt - value_of(last, x));
    return isinf(y) ? 100000.0 : y;
  }
  // One iteration of GSL's Brent minimiser on the state (xl, xu, xm, fm, v,
  // fv, w, fw, bd, be): the next probe u (a parabolic step, else golden
  // section).
  __device__ void gsl_brent_step() {
    z = xm;
    fz = fm;
    double dd = be, ee = bd;
    const double wl = z - xl, wu = xu - z;
    const double tolerance = 1.4901161193847656e-08 * fabs(z);
    double pp = 0, qq = 0, r = 0;
    const double mid = 0.5 * (xl + xu);
    if (fabs(ee) > tolerance) {
      r = (z - w) * (fz - fv);
      qq = (z - v) * (fz - fw);
      pp = (z - v) * qq - (z - w) * r;
      qq = 2 * (qq - r);
      if (qq > 0) pp = -pp; else qq = -qq;
      r = ee;
      ee = dd;
    }
    if (fabs(pp) < fabs(0.5 * qq * r) && pp < qq * wl && pp < qq * wu) {
      const double t2 = 2 * tolerance;
      dd = pp / qq;
      u = z + dd;
      if ((u - xl) < t2 || (xu - u) < t2) dd = (z < mid) ? tolerance : -tolerance;
    } else {
      ee = (z < mid) ? xu - z : -(z - xl);
      dd = 0.3819660 * ee;
    }
    if (fabs(dd) >= tolerance) u = z + dd;
    else u = z + ((dd > 0) ? tolerance : -tolerance);
    be = ee;
    bd = dd;
  }
  // The bracket and the (v, w, x) points after the value fval at u.
  __device__ void gsl_brent_update() {
    if (fval <= fz) {
      if (u < z) { xu = z; fu = fz; } else { xl = z; fl = fz; }
      v = w; fv = fw; w = z; fw = fz;
      xm = u; fm = fval;
    } else {
      if (u < z) { xl = u; fl = fval; } else { xu = u; fu = fval; }
      if (fval <= fw || w == z) { v = w; fv = fw; w = u; fw = fval; }
      else if (fval <= fv || v == z || v == w) { v = u; fv = fval; }
    }
  }

  __device__ void request(double pp, double dd, double xx, bool derivs) {
    req_p = (float)pp;
    req_d = (float)dd;
    req_x = (float)xx;
    req_derivs = derivs;
  }

  // set_pend_bl / set_dist_bl (three_tax.ml:38-45)
  __device__ void set_coord(int wh, double val) {
    if (wh == 0) {
      pend = val;
    } else {
      double pb = (dist + prox) - val;
      dist = val;
      prox = pb;
    }
  }

  // The Newton form needs the FP64 logL only at its start and end (it
  // compares evaluations by exact exponent differences), so it skips it here.
  __device__ void record(const EvalOut *res) {
    last = *res;
    if (optimizer != 1 || mode == 1) L_last = full(*res);
    n_evals++;
  }

  // The marginal likelihood as the reference computes it (pp_rule 1),
  // resumed after each evaluation like next(); only the kernels
  // instantiated with next<true>() contain it, so it adds nothing to the
  // trial kernels' site loops:
  // Three_tax.calc_marg_prob (three_tax.ml:169-215): the upper pendant
  // limit of find_upper_limit (three_tax.ml:124-159: Minimization.brent
  // with 10 iterations at tolerance 0.02 on |target - L - log prior|,
  // minimization.ml:24-41,83-101), then nested QNG to pp_rel -- the
  // distal integral over [0, cut] of the pendant integral over
  // [0, U] -- and on GSL_ETOL from either, U halved and the whole
  // integral retried, at most 10 times, after which the base
  // likelihood is the result.  A start-finder or iteration-limit
  // exception of the upper-limit search, or a non-finite objective (GSL's
  // EBADFUNC) -- which the reference does not catch there -- integrates to
  // max_pend, as its EINVAL does.
#define QNG_YIELD(label) \
  do {                   \
    qpc = label;         \
    return true;         \
    case label:;         \
  } while (0)
  __device__ __forceinline__ bool marg_qng() {
    switch (qpc) {
      case 0:
        qerr = 0;
        if (prior_kind == 1 && exp(log_prior(p)) == 0.0) {  // a zero prior: rewind (three_tax.ml:127-133)
          qU = p;
          for (k_srch = 0; k_srch < 1100 && !(exp(log_prior(qU * 0.5)) > exp(-10.0)); k_srch++) qU *= 0.5;
          goto QNG_RUN;
        }
        tgt = value_of(cur, p) - 10.0;
        left = p;
        right = max_pend;
        raw = p + (max_pend - p) / 2.0;
        if (left >= raw || raw >= right) { qerr = 1; qU = max_pend; goto QNG_RUN; }
        request(right, d, (float)cut - d, false);
        QNG_YIELD(40);
        righty = qng_objective(right);
        request(left, d, (float)cut - d, false);
        QNG_YIELD(41);
        lefty = qng_objective(left);
        smaller = lefty < righty ? left : right;
        miny = lefty <= righty ? lefty : righty;
        prevx = raw;
        for (iter = 1;; iter++) {
          request(prevx, d, (float)cut - d, false);
          QNG_YIELD(42);
          pv = qng_objective(prevx);
          if (pv < miny) break;
          if (fabs(prevx - smaller) < 0.02) { qU = smaller; goto QNG_RUN; }  // FoundMin
          if (iter > 10) { qerr = 2; qU = max_pend; goto QNG_RUN; }          // FindStartFailure
          prevx = 0.5 * (prevx + smaller);
        }
        xl = left; xu = right; xm = prevx;
        fl = lefty; fu = righty; fm = pv;
        if (!isfinite(fl) || !isfinite(fu) || !isfinite(fm)) { qerr = 5; qU = max_pend; goto QNG_RUN; }  // EBADFUNC
        if (!(fm < fl && fm < fu)) { qerr = 3; qU = max_pend; goto QNG_RUN; }  // GSL_EINVAL
        v = xl + 0.3819660 * (xu - xl);
        w = v;
        request(v, d, (float)cut - d, false);
        QNG_YIELD(43);
        fv = qng_objective(v);
        if (!isfinite(fv)) { qerr = 5; qU = max_pend; goto QNG_RUN; }
        fw = fv;
        bd = 0;
        be = 0;
        for (bstep = 1;; bstep++) {
          if (bstep > 10) { qerr = 4; qU = max_pend; goto QNG_RUN; }  // ExceededMaxIter
          gsl_brent_step();
          request(u, d, (float)cut - d, false);
          QNG_YIELD(44);
          fval = qng_objective(u);
          if (!isfinite(fval)) { qerr = 5; qU = max_pend; goto QNG_RUN; }
          gsl_brent_update();
          if (xu - xl < 0.02) { qU = xm; break; }
        }
      QNG_RUN:
        n_exc = 0;
      QNG_PERFORM:
        if (n_exc >= 10) {  // "integration did not converge after changing bounds 10 times"
          L_last = base;
          goto QNG_END;
        }
        oj = 0;
      QNG_OUTER:
        qd = fabs(cut) < 1e-5 ? 0.5 * cut : QngAcc::node(oj, 0.0, cut);
        ij = 0;
      QNG_INNER:
        qp = QngAcc::node(ij, 0.0, qU);
        request(qp, qd, cut - qd, false);
        QNG_YIELD(45);
        k_srch = qi.accept(ij, exp(full(last) - base + log_prior(qp)), 0.5 * qU, pp_rel);
        ij++;
        if (k_srch == 0) goto QNG_INNER;
        if (k_srch == 2) { n_exc++; qU *= 0.5; goto QNG_PERFORM; }
        if (fabs(cut) < 1e-5) {  // cut_bl =~ 0 (ppatteries.ml:96-97): the pendant integral alone
          L_last = base + log(qi.result);
          goto QNG_END;
        }
        k_srch = qo.accept(oj, qi.result, 0.5 * cut, pp_rel);
        oj++;
        if (k_srch == 0) goto QNG_OUTER;
        if (k_srch == 2) { n_exc++; qU *= 0.5; goto QNG_PERFORM; }
        L_last = base + log(qo.result / cut);
      QNG_END:
        status = isfinite(L_last) ? ST_OK : ST_FAILED;
        pend = p;
        dist = d;
        prox = (double)((float)cut - d);
        last = cur;
        return false;
    }
    return false;
  }
#undef QNG_YIELD


  template <bool QNG = false>
  __device__ __forceinline__ bool next(const EvalOut *res) {
    if (res) record(res);
    switch (pc) {
      case 0:
        status = ST_OK;
        attempt = 0;
        pend = pend0;
        dist = dist0;
        prox = cut - dist0;  // set_tt_edges (core.ml:225-239)
        if (mode == 1) {
          request(pend, dist, prox, true);
          PGB_YIELD(1);
          return false;
        }
        if (mode == 2) goto MARGINAL;
        if (optimizer == 1) goto NEWTON;
        // ---------------- Brent replica (three_tax.ml:48-83) ----------------
      BRENT_ATTEMPT:
        prev_pend = pend;
        prev_dist = dist;
        for (outer = 1;; outer++) {
          if (outer > 200) { status = ST_MAXITER; goto BRENT_DONE; }
          for (which = 0; which < 2; which++) {
            raw = which == 0 ? pend : dist;
            left = which == 0 ? 1e-8 : 0.0;
            right = which == 0 ? max_pend : dist + prox;
            if (left == right) { cres[which] = raw; continue; }
            // bisection_start_finder (minimization.ml:11-41)
            if (left >= raw || raw >= right) { status = ST_STARTFAIL; goto BRENT_DONE; }
            fx = right;
            set_coord(which, fx);
            request(pend, dist, prox, false);
            PGB_YIELD(10);
            righty = -L_last;
            fx = left;
            set_coord(which, fx);
            request(pend, dist, prox, false);
            PGB_YIELD(11);
            lefty = -L_last;
            smaller = lefty < righty ? left : right;
            miny = lefty <= righty ? lefty : righty;  // Stdlib.min
            prevx = raw;
            for (iter = 1;; iter++) {
              set_coord(which, prevx);
              request(pend, dist, prox, false);
              PGB_YIELD(12);
              pv = -L_last;
              if (pv < miny) break;
              if (fabs(prevx - smaller) < tol) { cres[which] = smaller; goto SEARCH_DONE; }  // FoundMin
              if (iter > 100) { status = ST_STARTFAIL; goto BRENT_DONE; }
              prevx = (prevx + smaller) / 2.;
            }
            // gsl_min_fminimizer_set (values of the finder's evaluations)
            xl = left; xu = right; xm = prevx;
            fl = lefty; fu = righty; fm = pv;
            if (!isfinite(fl) || !isfinite(fu) || !isfinite(fm)) { err = 1; goto BRENT_ERR; }
            if (xl > xu || xm >= xu || xm <= xl || fm >= fl || fm >= fu) { err = 1; goto BRENT_ERR; }
            v = xl + 0.3819660 * (xu - xl);
            w = v;
            set_coord(which, v);
            request(pend, dist, prox, false);
            PGB_YIELD(13);
            fv = -L_last;
            if (!isfinite(fv)) { err = 1; goto BRENT_ERR; }
            fw = fv;
            bd = 0;
            be = 0;
            for (bstep = 1;; bstep++) {
              if (bstep > 100) { status = ST_MAXITER; goto BRENT_DONE; }
              {
                // one GSL Brent iteration (parabolic step, else golden section)
                z = xm;
                fz = fm;
                double dd = be, ee = bd;
                double wl = z - xl, wu = xu - z;
                double tolerance = 1.4901161193847656e-08 * fabs(z);
                double pp = 0, qq = 0, r = 0;
                double mid = 0.5 * (xl + xu);
                if (fabs(ee) > tolerance) {
                  r = (z - w) * (fz - fv);
                  qq = (z - v) * (fz - fw);
                  pp = (z - v) * qq - (z - w) * r;
                  qq = 2 * (qq - r);
                  if (qq > 0) pp = -pp; else qq = -qq;
                  r = ee;
                  ee = dd;
                }
                if (fabs(pp) < fabs(0.5 * qq * r) && pp < qq * wl && pp < qq * wu) {
                  double t2 = 2 * tolerance;
                  dd = pp / qq;
                  u = z + dd;
                  if ((u - xl) < t2 || (xu - u) < t2) dd = (z < mid) ? tolerance : -tolerance;
                } else {
                  ee = (z < mid) ? xu - z : -(z - xl);
                  dd = 0.3819660 * ee;
                }
                if (fabs(dd) >= tolerance) u = z + dd;
                else u = z + ((dd > 0) ? tolerance : -tolerance);
                be = ee;
                bd = dd;
              }
              // A probe closer to z than the FP32 objective resolves is
              // decided by the adjoint's first-order model instead of by
              // two values equal to rounding.
              probe_dx = u - z;
              probe = fabs(probe_dx) < 1e-6;
              set_coord(which, u);
              request(pend, dist, prox, probe);
              PGB_YIELD(14);
              fval = probe ? fz - (double)last.g[which] * probe_dx : -L_last;
              if (!isfinite(fval)) { err = 1; goto BRENT_ERR; }
              if (fval <= fz) {
                if (u < z) { xu = z; fu = fz; } else { xl = z; fl = fz; }
                v = w; fv = fw; w = z; fw = fz;
                xm = u; fm = fval;
              } else {
                if (u < z) { xl = u; fl = fval; } else { xu = u; fu = fval; }
                if (fval <= fw || w == z) { v = w; fv = fw; w = u; fw = fval; }
                else if (fval <= fv || v == z || v == w) { v = u; fv = fval; }
              }
              if (xu - xl < tol) { cres[which] = xm; break; }
            }
          SEARCH_DONE:;
          }
          if (fabs(prev_pend - cres[0]) > tol || fabs(prev_dist - cres[1]) > tol) {
            prev_pend = cres[0];
            prev_dist = cres[1];
          } else {
            break;
          }
        }
        goto BRENT_DONE;
      BRENT_ERR:
        if (attempt == 0) {  // retry from the default branch lengths (core.ml:272-279)
          attempt = 1;
          pend = start_pend;
          dist = cut / 2.;
          prox = cut - cut / 2.;
          goto BRENT_ATTEMPT;
        }
        status = ST_FAILED;
      BRENT_DONE:
        if (n_evals == 0) {
          request(pend, dist, prox, false);
          PGB_YIELD(15);
        }
        return false;
        // ---------------- safeguarded projected Newton ----------------
      NEWTON:
        p = fminf(fmaxf((float)pend, 1e-8f), (float)max_pend);
        d = fminf(fmaxf((float)dist, 0.f), (float)cut);
        if (seeded) {  // the start point's evaluation is known (a refinement)
          seeded = false;
          last = seed;
        } else {
          request(p, d, (float)cut - d, true);
          PGB_YIELD(20);
        }
        cur = last;
        L_last = full(cur);
        if (!isfinite(cur.lm)) {
          if (attempt == 0) {
            attempt = 1;
            pend = start_pend;
            dist = cut / 2.;
            goto NEWTON;
          }
          status = ST_FAILED;
          pend = p; dist = d; prox = (double)((float)cut - d);
          return false;
        }
        allow = 1e-6f + 1e-9f * fabsf((float)L_last);
        stall = 0;
        for (it = 0; it < 60; it++) {
          {
            const float pmin = 1e-8f, pmax = (float)max_pend, dmax = (float)cut;
            float gp = cur.g[0], gd = cur.g[1], hpp = cur.h[0], hdd = cur.h[1], hpd = cur.h[2];
            bool free_p = !((p <= pmin && gp <= 0.f) || (p >= pmax && gp >= 0.f));
            bool free_d = (dmax > 0.f) && !((d <= 0.f && gd <= 0.f) || (d >= dmax && gd >= 0.f));
            if (!free_p && !free_d) break;
            sp = 0.f;
            sd = 0.f;
            float det = hpp * hdd - hpd * hpd;
            bool model = false;  // the step is a Newton step of a concave quadratic model
            if (free_p && free_d && hpp < 0.f && hdd < 0.f && det > 0.f) {
              sp = -(hdd * gp - hpd * gd) / det;
              sd = -(hpp * gd - hpd * gp) / det;
              model = true;
            } else {
              if (free_p) sp = hpp < 0.f ? -gp / hpp : copysignf(fmaxf(0.5f * p, 0.01f), gp);
              if (free_d) sd = hdd < 0.f ? -gd / hdd : copysignf(0.25f * dmax, gd);
              model = !(free_p && free_d) && (free_p ? hpp < 0.f : hdd < 0.f);
            }
            // Converged before stepping: the full Newton step would gain less
            // than the tolerance (g . s is twice the model's gain), so the
            // current point -- already evaluated -- is the result.
            if (model && gp * sp + gd * sd < newton_gain_tol() + allow) break;
            // Trust region: one factor for both coordinates, so the step
            // keeps the direction of the Newton (or diagonal) step, which is
            // an ascent direction.  Clipping each coordinate on its own can
            // turn it downhill -- on short edges the distal limit is tiny
            // while the pendant step is not -- and the line search then
            // shrinks it to nothing, iteration after iteration.
            float lim_p = fmaxf(2.f * p, 0.05f), lim_d = fmaxf(0.5f * dmax, 1e-12f);
            float f = 1.f;
            if (fabsf(sp) > lim_p) f = fminf(f, lim_p / fabsf(sp));
            if (fabsf(sd) > lim_d) f = fminf(f, lim_d / fabsf(sd));
            sp *= f;
            sd *= f;
            pred = gp * sp + gd * sd;
          }
          accepted = false;
          for (ls = 0; ls < 30; ls++) {
            np = fminf(fmaxf(p + sp, 1e-8f), (float)max_pend);
            nd = fminf(fmaxf(d + sd, 0.f), (float)cut);
            if (np == p && nd == d) break;
            request(np, nd, (float)cut - nd, true);
            PGB_YIELD(21);
            if (isfinite(last.lm) && dlogl(last, cur) >= -allow) {
              accepted = true;
              break;
            }
            sp *= 0.25f;
            sd *= 0.25f;
          }
          if (!accepted) break;
          {
            // three accepted steps in a row that gain less than the
            // evaluation's rounding allowance: the objective's noise floor
            float gain = dlogl(last, cur);
            float step = fmaxf(fabsf(np - p), fabsf(nd - d));
            p = np;
            d = nd;
            cur = last;
            stall = gain < allow ? stall + 1 : 0;
            if (fabsf(pred) < newton_gain_tol() + allow || step < 1e-9f || stall >= 3) break;
          }
          if (it == 59) status = ST_MAXITER;
        }
        pend = p;
        dist = d;
        prox = (double)((float)cut - d);
        last = cur;
        L_last = full(cur);
        return false;
        // ---------------- marginal likelihood (three_tax.ml:169-215) ----------------
        // log of (1/cut) int_0^cut int exp(L(p, d)) prior(p) dp dd, for the
        // posterior probabilities of core.ml:378-401.  The pendant range
        // ends where L + log prior has dropped 10 below its value at the
        // optimum (find_upper_limit, three_tax.ml:124-159; searched upward
        // and downward here), the distal range is the optimum +- 6 marginal
        // standard deviations of the Hessian's Gaussian (all of [0, cut]
        // when the Hessian is not negative definite); both are split at
        // the optimum and integrated by tensor Gauss-Legendre, kGlPoints
        // nodes per panel, in place of GSL's QNG.  A zero-length edge
        // integrates the pendant only, at the edge midpoint.
      MARGINAL:
        p = fminf(fmaxf((float)pend, 1e-8f), (float)max_pend);
        d = fminf(fmaxf((float)dist, 0.f), (float)cut);
        if (seeded) {
          seeded = false;
          last = seed;
        } else {
          request(p, d, (float)cut - d, true);
          PGB_YIELD(30);
        }
        cur = last;
        base = full(cur);
        pend = p;
        dist = d;
        prox = (double)((float)cut - d);
        if (!isfinite(base)) { status = ST_FAILED; L_last = base; return false; }
        if (pp_rule == 1) {  // only kernels built with QNG carry that computation
          if (!QNG) { status = ST_FAILED; L_last = NAN; return false; }
          qpc = 0;
          goto QNG_STEP;
        }
        tgt = value_of(cur, p) - 10.0;
        {
          const double hpp = cur.h[0], hdd = cur.h[1], hpd = cur.h[2];
          const double det = hpp * hdd - hpd * hpd;
          const bool nd = hpp < 0.0 && hdd < 0.0 && det > 0.0;
          sig_p = nd ? sqrt(-hdd / det) : 0.05;
          sig_d = nd ? sqrt(-hpp / det) : 1e30;
        }
        // upper pendant limit
        stp = fmax(sig_p, 1e-4);
        lo_b = p;
        hi_b = p;
        for (k_srch = 0; k_srch < 60; k_srch++) {
          qp = fmin(hi_b + stp, max_pend);
          if (qp <= hi_b) break;  // at max_pend
          request(qp, d, (float)cut - d, false);
          PGB_YIELD(31);
          if (!(value_of(last, qp) > tgt)) { lo_b = hi_b; hi_b = qp; break; }
          hi_b = qp;
          lo_b = qp;
          stp *= 2.0;
        }
        for (k_srch = 0; k_srch < 6 && hi_b > lo_b; k_srch++) {  // refine the crossing
          qp = 0.5 * (lo_b + hi_b);
          request(qp, d, (float)cut - d, false);
          PGB_YIELD(32);
          if (!(value_of(last, qp) > tgt)) hi_b = qp;
          else lo_b = qp;
        }
        ppan[2] = hi_b;
        // lower pendant limit
        stp = fmax(sig_p, 1e-4);
        lo_b = p;
        hi_b = p;
        for (k_srch = 0; k_srch < 60; k_srch++) {
          qp = fmax(lo_b - stp, 0.0);
          if (qp >= lo_b) break;  // at 0
          request(fmax(qp, 1e-8), d, (float)cut - d, false);
          PGB_YIELD(33);
          if (!(value_of(last, qp) > tgt)) { hi_b = lo_b; lo_b = qp; break; }
          lo_b = qp;
          hi_b = qp;
          stp *= 2.0;
        }
        for (k_srch = 0; k_srch < 6 && hi_b > lo_b; k_srch++) {
          qp = 0.5 * (lo_b + hi_b);
          request(qp, d, (float)cut - d, false);
          PGB_YIELD(34);
          if (!(value_of(last, qp) > tgt)) lo_b = qp;
          else hi_b = qp;
        }
        ppan[0] = lo_b;
        ppan[1] = p;
        // distal range
        if (cut <= 1e-10) {
          n_dpan = 0;  // zero-length edge: the pendant integral alone, at cut / 2
        } else {
          dpan[0] = fmax(0.0, (double)d - 6.0 * sig_d);
          dpan[1] = d;
          dpan[2] = fmin(cut, (double)d + 6.0 * sig_d);
          n_dpan = 2;
        }
        acc_out = 0.0;
        for (jpan = 0; jpan < (n_dpan ? n_dpan : 1); jpan++) {
          if (n_dpan && !(dpan[jpan + 1] > dpan[jpan])) continue;
          for (jd = 0; jd < (n_dpan ? kGlPoints : 1); jd++) {
            if (n_dpan) {
              const double half = 0.5 * (dpan[jpan + 1] - dpan[jpan]);
              qd = dpan[jpan] + half * (1.0 + gl[jd]);
              wd = half * gl[kGlPoints + jd];
            } else {
              qd = 0.5 * cut;
              wd = 1.0;
            }
            acc_in = 0.0;
            for (ipan = 0; ipan < 2; ipan++) {
              if (!(ppan[ipan + 1] > ppan[ipan])) continue;
              for (ip = 0; ip < kGlPoints; ip++) {
                {
                  const double half = 0.5 * (ppan[ipan + 1] - ppan[ipan]);
                  qp = ppan[ipan] + half * (1.0 + gl[ip]);
                }
                request(fmax(qp, 1e-8), qd, cut - qd, false);
                PGB_YIELD(35);
                acc_in += 0.5 * (ppan[ipan + 1] - ppan[ipan]) * gl[kGlPoints + ip] *
                          exp(full(last) - base + log_prior(qp));
              }
            }
            acc_out += wd * acc_in;
          }
        }
        L_last = base + log(n_dpan ? acc_out / cut : acc_out);
        status = isfinite(L_last) ? ST_OK : ST_FAILED;
        last = cur;
        return false;
      case 46:  // the reference's computation (marg_qng), resumed after each evaluation
      QNG_STEP:
        if (QNG && marg_qng()) {
          pc = 46;
          return true;
        }
        return false;
      default:
        return false;
    }
  }
};
#undef PGB_YIELD

// ---------------------------------------------------------------------------
// Per-evaluation tables, shared by the CTA and the warp kernels.  Threads
// i0, i0 + stride, ... of the group fill them; the caller synchronises the
// group between trial_exps and trial_tables and before the sites read them.
// ---------------------------------------------------------------------------

// exp / expm1 of rate * lambda * t for t = dist, prox, pend: E, Em1 [3][NM][K]
__device__ __forceinline__ void trial_exps(const TrialSmem &sm, int NM, int K, const Ctrl &ctl, int i0, int stride) {
  for (int i = i0; i < 3 * NM * K; i += stride) {
    int wh = i / (NM * K), mk = i - wh * NM * K;
    float t = wh == 0 ? ctl.dist : (wh == 1 ? ctl.prox : ctl.pend);
    float a = sm.Lr[mk] * t;
    sm.E[i] = expf(a);
    sm.Em1[i] = expm1f(a);
  }
}

// P(t) = I + X diag(expm1(r lambda t)) X^-T for the distal and proximal
// lengths, its first and second derivatives, and the statd-weighted evolved
// query vectors Z (and d/dpend, d2/dpend2) of every character code.
__device__ __forceinline__ void trial_tables(const TrialSmem &sm, const float *W, int NM, int nc, int ncz, int K,
                                             bool derivs, int i0, int stride, bool mats = true) {
  const int nmat = NM * K * K;
  for (int i = i0; i < (mats ? 2 * nmat : 0); i += stride) {
    int wh = i / nmat, r = i - wh * nmat;
    int m = r / (K * K), ij = r - m * K * K;
    int ii = ij / K, jj = ij - ii * K;
    const float *w = W + (long)ij * K;
    const float *em = sm.Em1 + (wh * NM + m) * K;
    float a = (ii == jj) ? 1.f : 0.f;
#pragma unroll 4
    for (int k = 0; k < K; k++) a = fmaf(w[k], em[k], a);
    (wh == 0 ? sm.Md : sm.Mp)[r] = a;
    if (derivs) {
      const float *e = sm.E + (wh * NM + m) * K;
      const float *lr = sm.Lr + m * K;
      float a1 = 0.f, a2 = 0.f;
#pragma unroll 4
      for (int k = 0; k < K; k++) {
        float t1 = w[k] * lr[k] * e[k];
        a1 += t1;
        a2 = fmaf(t1, lr[k], a2);
      }
      (wh == 0 ? sm.Md1 : sm.Mp1)[r] = a1;
      (wh == 0 ? sm.Md2 : sm.Mp2)[r] = a2;
    }
  }
  // Z rows of codes 0 .. ncz - 1 only (ncz = the primary states when the
  // query has no ambiguity character); the table keeps its nc-row stride
  const int nz = NM * ncz * K;
  for (int j = i0; j < nz; j += stride) {
    int m = j / (ncz * K), ck = j - m * ncz * K;
    int code = ck / K, ii = ck - code * K;
    const int i = (m * nc + code) * K + ii;
    const float *x = sm.X + ii * K;
    const float *lt = sm.Lt + code * K;
    const float *em = sm.Em1 + (2 * NM + m) * K;
    float a = sm.lv[code * K + ii];
#pragma unroll 4
    for (int k = 0; k < K; k++) a = fmaf(x[k] * em[k], lt[k], a);
    float pi = sm.statd[ii];
    sm.Z[i] = pi * a;
    if (derivs) {
      const float *e = sm.E + (2 * NM + m) * K;
      const float *lr = sm.Lr + m * K;
      float a1 = 0.f, a2 = 0.f;
#pragma unroll 4
      for (int k = 0; k < K; k++) {
        float t1 = x[k] * lr[k] * e[k] * lt[k];
        a1 += t1;
        a2 = fmaf(t1, lr[k], a2);
      }
      sm.Z1[i] = pi * a1;
      sm.Z2[i] = pi * a2;
    }
  }
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------

// per-site likelihood and its derivatives -> running (mantissa, exponent)
// product and derivative sums of the thread
struct SiteAcc {
  float m;
  int e;
  float gp, gd, hpp, hdd, hpd;
  __device__ void init() { m = 1.f; e = 0; gp = gd = hpp = hdd = hpd = 0.f; }
  __device__ __forceinline__ void add(float u, float ud, float udd, float up, float upp, float upd, bool derivs) {
    // u = 2^eu * mu with mu in [0.5, 1): read from the bits for positive
    // normal u; zero, subnormal, negative and non-finite u take frexpf and a
    // full division, so a zero or NaN site still reaches the product.
    const unsigned bu = __float_as_uint(u);
    float mu, inv = 0.f;
    if ((bu >> 23) - 1u < 254u) {
      e += (int)(bu >> 23) - 126;
      mu = __uint_as_float((bu & 0x007fffffu) | 0x3f000000u);
      if (derivs) inv = __fdividef(1.f, u);
    } else {
      int eu;
      mu = frexpf(u, &eu);
      e += eu;
      if (derivs) inv = 1.f / u;
    }
    // m, mu in [0.5, 1): the product is a positive normal number or zero
    m *= mu;
    const unsigned bm = __float_as_uint(m);
    if (bm != 0u && (bm >> 23) < 255u) {
      e += (int)(bm >> 23) - 126;
      m = __uint_as_float((bm & 0x007fffffu) | 0x3f000000u);
    }
    if (derivs) {
      float lp = up * inv, ld = ud * inv;
      gp += lp;
      gd += ld;
      hpp += upp * inv - lp * lp;
      hdd += udd * inv - ld * ld;
      hpd += upd * inv - lp * ld;
    }
  }
};

// Sites of the DNA Gamma-mixture model: rates outer, the rate's transition
// matrices held in registers, the thread's sites inner.
template <int T, bool DER>
__device__ __forceinline__ void sites_dna_gmix(const TrialCtx &c, const TrialSmem &sm, int q, int node, int Sq,
                                               SiteAcc &acc) {
  constexpr int K = 4;
  const int tid = threadIdx.x, nc = c.ncode;
  const float *gdb = c.darr + (long)node * c.S * c.RP * K;
  const float *gpb = c.parr + (long)node * c.S * c.RP * K;
  for (int base = 0; base < Sq; base += 4 * T) {
    float a0[4], ad[4], add[4], ap[4], app[4], apd[4];
#pragma unroll
    for (int j = 0; j < 4; j++) a0[j] = ad[j] = add[j] = ap[j] = app[j] = apd[j] = 0.f;
    for (int r = 0; r < c.RP; r++) {
      float md[16], mp[16], md1[DER ? 16 : 1], md2[DER ? 16 : 1], mp1[DER ? 16 : 1], mp2[DER ? 16 : 1];
#pragma unroll
      for (int t = 0; t < 16; t += 4) {
        float4 a = *reinterpret_cast<const float4 *>(sm.Md + r * 16 + t);
        float4 b = *reinterpret_cast<const float4 *>(sm.Mp + r * 16 + t);
        md[t] = a.x; md[t + 1] = a.y; md[t + 2] = a.z; md[t + 3] = a.w;
        mp[t] = b.x; mp[t + 1] = b.y; mp[t + 2] = b.z; mp[t + 3] = b.w;
        if (DER) {
          float4 c1 = *reinterpret_cast<const float4 *>(sm.Md1 + r * 16 + t);
          float4 c2 = *reinterpret_cast<const float4 *>(sm.Md2 + r * 16 + t);
          float4 e1 = *reinterpret_cast<const float4 *>(sm.Mp1 + r * 16 + t);
          float4 e2 = *reinterpret_cast<const float4 *>(sm.Mp2 + r * 16 + t);
          md1[t] = c1.x; md1[t + 1] = c1.y; md1[t + 2] = c1.z; md1[t + 3] = c1.w;
          md2[t] = c2.x; md2[t + 1] = c2.y; md2[t + 2] = c2.z; md2[t + 3] = c2.w;
          mp1[t] = e1.x; mp1[t + 1] = e1.y; mp1[t + 2] = e1.z; mp1[t + 3] = e1.w;
          mp2[t] = e2.x; mp2[t + 1] = e2.y; mp2[t + 2] = e2.z; mp2[t + 3] = e2.w;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        int i = base + tid + j * T;
        if (i < Sq) {
          int code = sm.code[i];
          float4 D4, P4;
          if (c.smem_win) {
            D4 = *reinterpret_cast<const float4 *>(sm.D + ((long)r * c.cap + i) * K);
            P4 = *reinterpret_cast<const float4 *>(sm.P + ((long)r * c.cap + i) * K);
          } else {
            long s = c.reind[(long)q * c.S + i];
            D4 = __ldg(reinterpret_cast<const float4 *>(gdb + (s * c.RP + r) * K));
            P4 = __ldg(reinterpret_cast<const float4 *>(gpb + (s * c.RP + r) * K));
          }
          const float dv[4] = {D4.x, D4.y, D4.z, D4.w}, pv[4] = {P4.x, P4.y, P4.z, P4.w};
          float4 Z4 = *reinterpret_cast<const float4 *>(sm.Z + (r * nc + code) * K);
          const float z[4] = {Z4.x, Z4.y, Z4.z, Z4.w};
          float z1[4], z2[4];
          if (DER) {
            float4 a = *reinterpret_cast<const float4 *>(sm.Z1 + (r * nc + code) * K);
            float4 b = *reinterpret_cast<const float4 *>(sm.Z2 + (r * nc + code) * K);
            z1[0] = a.x; z1[1] = a.y; z1[2] = a.z; z1[3] = a.w;
            z2[0] = b.x; z2[1] = b.y; z2[2] = b.z; z2[3] = b.w;
          }
#pragma unroll
          for (int ii = 0; ii < 4; ii++) {
            float x = 0.f, y = 0.f;
#pragma unroll
            for (int jj = 0; jj < 4; jj++) {
              x = fmaf(md[ii * 4 + jj], dv[jj], x);
              y = fmaf(mp[ii * 4 + jj], pv[jj], y);
            }
            float xy = x * y;
            a0[j] = fmaf(z[ii], xy, a0[j]);
            if (DER) {
              float x1 = 0.f, x2 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
              for (int jj = 0; jj < 4; jj++) {
                x1 = fmaf(md1[ii * 4 + jj], dv[jj], x1);
                x2 = fmaf(md2[ii * 4 + jj], dv[jj], x2);
                y1 = fmaf(mp1[ii * 4 + jj], pv[jj], y1);
                y2 = fmaf(mp2[ii * 4 + jj], pv[jj], y2);
              }
              float aa = x1 * y - x * y1;
              float bb = x2 * y - 2.f * x1 * y1 + x * y2;
              ad[j] = fmaf(z[ii], aa, ad[j]);
              add[j] = fmaf(z[ii], bb, add[j]);
              ap[j] = fmaf(z1[ii], xy, ap[j]);
              app[j] = fmaf(z2[ii], xy, app[j]);
              apd[j] = fmaf(z1[ii], aa, apd[j]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (base + tid + j * T < Sq) acc.add(a0[j], ad[j], add[j], ap[j], app[j], apd[j], DER);
  }
}

// Generic sites: any K, Gamma mixture or per-site CAT category matrices read
// from shared memory.
template <int K, int T, bool DER>
__device__ __forceinline__ void sites_generic(const TrialCtx &c, const TrialSmem &sm, int q, int node, int Sq,
                                              SiteAcc &acc) {
  const int tid = threadIdx.x, nc = c.ncode;
  const float *gdb = c.darr + (long)node * c.S * c.RP * K;
  const float *gpb = c.parr + (long)node * c.S * c.RP * K;
  for (int i = tid; i < Sq; i += T) {
    int code = sm.code[i];
    float u = 0.f, ud = 0.f, udd = 0.f, up = 0.f, upp = 0.f, upd = 0.f;
    long s = c.smem_win ? 0 : (long)c.reind[(long)q * c.S + i];
    for (int r = 0; r < c.RP; r++) {
      int m = c.gcat ? sm.cat[i] : r;
      float dv[K], pv[K];
      const float *ds = c.smem_win ? sm.D + ((long)r * c.cap + i) * K : gdb + (s * c.RP + r) * K;
      const float *ps = c.smem_win ? sm.P + ((long)r * c.cap + i) * K : gpb + (s * c.RP + r) * K;
#pragma unroll
      for (int k = 0; k < K; k += 4) {
        float4 a = *reinterpret_cast<const float4 *>(ds + k);
        float4 b = *reinterpret_cast<const float4 *>(ps + k);
        dv[k] = a.x; dv[k + 1] = a.y; dv[k + 2] = a.z; dv[k + 3] = a.w;
        pv[k] = b.x; pv[k + 1] = b.y; pv[k + 2] = b.z; pv[k + 3] = b.w;
      }
      const float *Md = sm.Md + m * K * K, *Mp = sm.Mp + m * K * K;
      const float *z = sm.Z + (m * nc + code) * K;
#pragma unroll(K <= 4 ? K : 1)
      for (int ii = 0; ii < K; ii++) {
        float x = 0.f, y = 0.f;
#pragma unroll
        for (int jj = 0; jj < K; jj++) {
          x = fmaf(Md[ii * K + jj], dv[jj], x);
          y = fmaf(Mp[ii * K + jj], pv[jj], y);
        }
        float xy = x * y;
        u = fmaf(z[ii], xy, u);
        if (DER) {
          const float *Md1 = sm.Md1 + m * K * K, *Md2 = sm.Md2 + m * K * K;
          const float *Mp1 = sm.Mp1 + m * K * K, *Mp2 = sm.Mp2 + m * K * K;
          float x1 = 0.f, x2 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
          for (int jj = 0; jj < K; jj++) {
            x1 = fmaf(Md1[ii * K + jj], dv[jj], x1);
            x2 = fmaf(Md2[ii * K + jj], dv[jj], x2);
            y1 = fmaf(Mp1[ii * K + jj], pv[jj], y1);
            y2 = fmaf(Mp2[ii * K + jj], pv[jj], y2);
          }
          float z1 = sm.Z1[(m * nc + code) * K + ii], z2 = sm.Z2[(m * nc + code) * K + ii];
          float aa = x1 * y - x * y1;
          float bb = x2 * y - 2.f * x1 * y1 + x * y2;
          ud = fmaf(z[ii], aa, ud);
          udd = fmaf(z[ii], bb, udd);
          up = fmaf(z1, xy, up);
          upp = fmaf(z2, xy, upp);
          upd = fmaf(z1, aa, upd);
        }
      }
    }
    acc.add(u, ud, udd, up, upp, upd, DER);
  }
}

// Model constants of the CTA form, once per CTA.
template <int K, int T>
__device__ __forceinline__ void trial_cta_setup(const TrialCtx &c, const TrialSmem &sm) {
  const int tid = threadIdx.x, NM = c.NM, nc = c.ncode;
  for (int i = tid; i < K * K; i += T) sm.X[i] = c.X[i];
  if (K == 4)
    for (int i = tid; i < K * K * K; i += T) sm.W[i] = c.W[i];
  for (int i = tid; i < nc * K; i += T) { sm.Lt[i] = c.Lt[i]; sm.lv[i] = c.lvf[i]; }
  for (int i = tid; i < NM * K; i += T) sm.Lr[i] = c.rates[i / K] * c.lam[i % K];
  if (tid < K) sm.statd[tid] = c.statd[tid];
}

// One trial by the CTA (after trial_cta_setup); every thread returns the
// same result.
template <int K, int T, bool QNG = false>
__device__ TrialRes trial_cta(const TrialCtx &c, const TrialSmem &sm, const TrialIn &tr) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = tr.q, node = tr.node;
  const int Sq = c.qlen[q];
  const int NM = c.NM, nc = c.ncode;
  __syncthreads();  // the previous trial's readers of the shared state are done
  // ---- prologue: the query's sites of darr / parr ----
  long long esum = 0;
  const long qo = (long)q * c.S;
  for (int i = tid; i < Sq; i += T) {
    int s = c.reind[qo + i];
    sm.code[i] = c.mcode[qo + i];
    if (c.gcat) sm.cat[i] = c.site_cat[s];
    long go = ((long)node * c.S + s);
    esum += (long long)c.dexp[go] + (long long)c.pexp[go];
    if (c.smem_win) {
      for (int r = 0; r < c.RP; r++) {
        const float *ds = c.darr + (go * c.RP + r) * K;
        const float *ps = c.parr + (go * c.RP + r) * K;
        float *dd = sm.D + ((long)r * c.cap + i) * K;
        float *pd = sm.P + ((long)r * c.cap + i) * K;
#pragma unroll
        for (int k = 0; k < K; k += 4) {
          *reinterpret_cast<float4 *>(dd + k) = __ldg(reinterpret_cast<const float4 *>(ds + k));
          *reinterpret_cast<float4 *>(pd + k) = __ldg(reinterpret_cast<const float4 *>(ps + k));
        }
      }
    }
  }
  esum = warp_sum_ll(esum);
  __shared__ long long s_esum[(T / 32)];
  if (lane == 0) s_esum[warp] = esum;
  __syncthreads();
  long long etot = 0;
  for (int i = 0; i < (T / 32); i++) etot += s_esum[i];

  Optimiser opt;
  if (warp == 0) {
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
    // ---- warp 0: next point, exp factors ----
    if (warp == 0) {
      bool more = opt.template next<QNG>(ev == 0 ? nullptr : &res);
      if (lane == 0) {
        sm.ctrl->cmd = more ? (opt.req_derivs ? 2 : 1) : 0;
        sm.ctrl->pend = opt.req_p;
        sm.ctrl->dist = opt.req_d;
        sm.ctrl->prox = opt.req_x;
      }
    }
    __syncthreads();  // A
    const Ctrl ctl = *sm.ctrl;
    if (ctl.cmd == 0) break;
    const bool derivs = ctl.cmd == 2;
    trial_exps(sm, NM, K, ctl, tid, T);
    __syncthreads();  // A2: exp factors
    trial_tables(sm, K == 4 ? sm.W : c.W, NM, nc, c.qamb[q] > 0 ? nc : c.prim, K, derivs, tid, T);
    __syncthreads();  // B
    // ---- sites ----
    SiteAcc acc;
    acc.init();
    if (K == 4 && !c.gcat) {
      if (derivs) sites_dna_gmix<T, true>(c, sm, q, node, Sq, acc);
      else sites_dna_gmix<T, false>(c, sm, q, node, Sq, acc);
    } else {
      if (derivs) sites_generic<K, T, true>(c, sm, q, node, Sq, acc);
      else sites_generic<K, T, false>(c, sm, q, node, Sq, acc);
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
    __syncthreads();  // C
    if (warp == 0) {
      // lanes 0..warps-1 hold one warp's partials; shuffle tree
      bool have = lane < (T / 32);
      float mt = have ? sm.red[lane * 8] : 1.f;
      int et = have ? sm.redi[lane] : 0;
      float sg[5];
#pragma unroll
      for (int k = 0; k < 5; k++) sg[k] = have ? sm.red[lane * 8 + 1 + k] : 0.f;
#pragma unroll
      for (int o = (T / 32) / 2; o > 0; o >>= 1) {
        float mo = __shfl_xor_sync(0xffffffffu, mt, o);
        int eo = __shfl_xor_sync(0xffffffffu, et, o);
        mt *= mo;
        et += eo;
        int em;
        mt = frexpf(mt, &em);
        et += em;
#pragma unroll
        for (int k = 0; k < 5; k++) sg[k] += __shfl_xor_sync(0xffffffffu, sg[k], o);
      }
      mt = __shfl_sync(0xffffffffu, mt, 0);
      et = __shfl_sync(0xffffffffu, et, 0);
#pragma unroll
      for (int k = 0; k < 5; k++) sg[k] = __shfl_sync(0xffffffffu, sg[k], 0);
      res.ex = et;
      res.lm = logf(mt);
      res.g[0] = sg[0]; res.g[1] = sg[1];
      res.h[0] = sg[2]; res.h[1] = sg[3]; res.h[2] = sg[4];
    }
  }
  if (tid == 0) {
    TrialRes r;
    r.like = opt.L_last;
    r.pend = opt.pend;
    r.dist = opt.dist;
    r.der[0] = opt.last.g[0]; r.der[1] = opt.last.g[1];
    r.der[2] = opt.last.h[0]; r.der[3] = opt.last.h[1]; r.der[4] = opt.last.h[2];
    r.der[5] = 0;
    r.status = opt.status;
    r.last = opt.last;
    r.n_evals = opt.n_evals;
    *sm.res = r;
    if (c.stats) {
      atomicAdd(&c.stats[0], (unsigned long long)opt.n_evals);
      atomicAdd(&c.stats[1], (unsigned long long)opt.n_evals * (unsigned long long)Sq);
    }
  }
  __syncthreads();
  return *sm.res;
}

template <int K, int T, bool QNG = false>
__global__ void __launch_bounds__(T, 1) k_trials(TrialCtx c, const TrialIn *__restrict__ trials,
                                                 const int *__restrict__ order, int n, TrialRes *out) {
  extern __shared__ __align__(16) char t_smem[];
  if (blockIdx.x >= n) return;
  const int ti = order ? order[blockIdx.x] : blockIdx.x;
  const TrialSmem sm = carve(t_smem, c.cap, c.smem_win, c.RP, K, c.NM, c.ncode);
  trial_cta_setup<K, T>(c, sm);
  const TrialRes r = trial_cta<K, T, QNG>(c, sm, trials[ti]);
  if (threadIdx.x == 0) out[ti] = r;
}
