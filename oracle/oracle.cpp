// ORACLE -- test infrastructure only.  FP64 CPU restatement of pplacer's
// placement-likelihood path, used by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py as the checker.  The product (pplacer_gb300/)
// never links or calls this file.
//
// Each block cites the reference file:line it restates (paths relative to the
// pplacer source tree).  The third-party arithmetic pplacer takes from GSL
// (ocaml gsl 1.25.0 over libgsl 2.7, opam-requirements.txt:6) is restated
// from the published algorithms: Brent's minimiser with GSL's conventions
// (R. P. Brent, "Algorithms for Minimization without Derivatives", 1973,
// ch. 5), a cyclic Jacobi symmetric eigensolver in place of gsl_eigen_symmv,
// and the regularised incomplete gamma function by series / continued
// fraction in place of gsl_sf_gamma_inc_P and gsl_cdf_gamma_Pinv.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// L0: linear_c.c kernels (pplacer_src/linear_c.c).  Loop and summation order
// follow the reference so that results agree to the last bit when built with
// -ffp-contract=off.
// ---------------------------------------------------------------------------

// dst[s,i] = sum_j a[i,j] b[s,j]                          (linear_c.c:29-90)
static void gemmish(double *dst, const double *a, const double *b, int n_sites, int n_states) {
  for (int s = 0; s < n_sites; s++) {
    const double *bs = b + (size_t)s * n_states;
    for (int i = 0; i < n_states; i++) {
      const double *ai = a + (size_t)i * n_states;
      double acc = 0;
      for (int j = 0; j < n_states; j++) acc += ai[j] * bs[j];
      dst[(size_t)s * n_states + i] = acc;
    }
  }
}

// dst[i,j] = sum_k lambda[k] u[i,k] uit[j,k]              (linear_c.c:92-146)
static void dediagonalize(double *dst, const double *u, const double *lambda, const double *uit, int n) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double acc = 0;
      for (int k = 0; k < n; k++) acc += lambda[k] * u[i * n + k] * uit[j * n + k];
      dst[i * n + j] = acc;
    }
}

// sum_s log sum_k statd_k x y z                           (linear_c.c:170-216)
static double mat_log_like3(const double *statd, const double *x, const double *y, const double *z,
                            int n_sites, int n_states) {
  double ll = 0;
  for (int s = 0; s < n_sites; s++) {
    double u = 0;
    for (int k = 0; k < n_states; k++) u += statd[k] * x[k] * y[k] * z[k];
    ll += std::log(u);
    x += n_states; y += n_states; z += n_states;
  }
  return ll;
}

// dst = x * y elementwise                      (linear_c.c:218-230, 426-441)
static void pairwise_prod(double *dst, const double *x, const double *y, size_t n) {
  for (size_t i = 0; i < n; i++) dst[i] = x[i] * y[i];
}

// dst[.., s, k] = statd_k a b                  (linear_c.c:232-249, 443-463)
static void statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                size_t n_rows, int n_states) {
  for (size_t s = 0; s < n_rows; s++)
    for (int k = 0; k < n_states; k++) {
      *dst = statd[k] * (*a) * (*b);
      dst++; a++; b++;
    }
}

// sum_{s: mask} log sum_k x y                             (linear_c.c:251-296)
static double mat_masked_logdot(const double *x, const double *y, const uint16_t *mask, int n_sites,
                                int n_states) {
  double ll = 0;
  for (int s = 0; s < n_sites; s++) {
    if (mask[s]) {
      double u = 0;
      for (int k = 0; k < n_states; k++) u += x[k] * y[k];
      ll += std::log(u);
    }
    x += n_states; y += n_states;
  }
  return ll;
}

// sum_{s in [first,last]} log sum_k x y                   (linear_c.c:298-340)
static double mat_bounded_logdot(const double *x, const double *y, int first, int last, int n_states) {
  double ll = 0;
  x += (size_t)first * n_states; y += (size_t)first * n_states;
  for (int s = 0; s < 1 + last - first; s++) {
    double u = 0;
    for (int k = 0; k < n_states; k++) u += x[k] * y[k];
    x += n_states; y += n_states;
    ll += std::log(u);
  }
  return ll;
}

// sum_s log(sum_r sum_k statd x y z) - S log R            (linear_c.c:367-424)
static double ten_log_like3(const double *statd, const double *x, const double *y, const double *z,
                            double *util, int n_rates, int n_sites, int n_states) {
  for (int s = 0; s < n_sites; s++) util[s] = 0.0;
  for (int r = 0; r < n_rates; r++)
    for (int s = 0; s < n_sites; s++) {
      for (int k = 0; k < n_states; k++) util[s] += statd[k] * x[k] * y[k] * z[k];
      x += n_states; y += n_states; z += n_states;
    }
  double ll = 0;
  for (int s = 0; s < n_sites; s++) ll += std::log(util[s]);
  ll -= ((float)n_sites) * std::log((double)(float)n_rates);
  return ll;
}

// masked Gmix logdot                                      (linear_c.c:465-539)
static double ten_masked_logdot(const double *x, const double *y, const uint16_t *mask, double *util,
                                int n_rates, int n_sites, int n_states) {
  for (int s = 0; s < n_sites; s++) util[s] = 0.0;
  for (int r = 0; r < n_rates; r++) {
    const double *xp = x + (size_t)r * n_sites * n_states, *yp = y + (size_t)r * n_sites * n_states;
    for (int s = 0; s < n_sites; s++) {
      if (mask[s])
        for (int k = 0; k < n_states; k++) util[s] += xp[k] * yp[k];
      xp += n_states; yp += n_states;
    }
  }
  double ll = 0;
  int n_used = 0;
  for (int s = 0; s < n_sites; s++)
    if (mask[s]) { ll += std::log(util[s]); n_used++; }
  ll -= ((float)n_used) * std::log((double)(float)n_rates);
  return ll;
}

// windowed Gmix logdot                                    (linear_c.c:541-605)
static double ten_bounded_logdot(const double *x, const double *y, int first, int last, double *util,
                                 int n_rates, int n_sites, int n_states) {
  int n_used = 1 + last - first;
  for (int s = 0; s < n_used; s++) util[s] = 0.0;
  for (int r = 0; r < n_rates; r++) {
    size_t boost = (size_t)r * n_sites * n_states + (size_t)first * n_states;
    const double *xp = x + boost, *yp = y + boost;
    for (int s = 0; s < n_used; s++) {
      for (int k = 0; k < n_states; k++) util[s] += xp[k] * yp[k];
      xp += n_states; yp += n_states;
    }
  }
  double ll = 0;
  for (int s = 0; s < n_used; s++) ll += std::log(util[s]);
  ll -= ((float)n_used) * std::log((double)(float)n_rates);
  return ll;
}

// ---------------------------------------------------------------------------
// Symmetric eigendecomposition (stands in for gsl_eigen_symmv,
// common_src/linear_utils.ml:206-208): cyclic Jacobi rotations until the
// off-diagonal mass is below machine precision.  a (n x n) is destroyed;
// eigenvalues to l, eigenvectors as the columns of v.
// ---------------------------------------------------------------------------
static void jacobi_eigen(std::vector<double> a, int n, std::vector<double> &l, std::vector<double> &v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) v[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0, tot = 0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        tot += a[i * n + j] * a[i * n + j];
        if (i != j) off += a[i * n + j] * a[i * n + j];
      }
    if (off <= 1e-34 * tot || off == 0) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = a[p * n + q];
        if (apq == 0) continue;
        double app = a[p * n + p], aqq = a[q * n + q];
        double theta = (aqq - app) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; k++) {  // A <- A J (columns p, q)
          double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {  // A <- J^T A (rows p, q)
          double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  l.resize(n);
  for (int i = 0; i < n; i++) l[i] = a[i * n + i];
}

static std::vector<double> matmul(const std::vector<double> &a, const std::vector<double> &b, int n) {
  std::vector<double> c((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double acc = 0;
      for (int k = 0; k < n; k++) acc += a[i * n + k] * b[k * n + j];
      c[i * n + j] = acc;
    }
  return c;
}

// ---------------------------------------------------------------------------
// Diagd (pplacer_src/diagd.ml)
// ---------------------------------------------------------------------------
struct Diagd {
  int n = 0;
  std::vector<double> x, l, xit;  // x diag(l) x^-1 = B D ; xit = x^-T
};

static double safe_invert(double v) { return v == 0. ? 1. : 1. / v; }  // diagd.ml:118

// of_d_b: X = D^-1/2 U, Xit = D^1/2 U with U L U^T = D^1/2 B D^1/2  (diagd.ml:123-132)
static Diagd of_d_b(const std::vector<double> &d, const std::vector<double> &b, int n) {
  for (int i = 0; i < n; i++)
    if (!(d[i] >= 0)) throw std::runtime_error("negative element in the diagonal of a DB matrix!");
  std::vector<double> droot(n), dm((size_t)n * n, 0.0), dmi((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    droot[i] = std::sqrt(d[i]);
    dm[i * n + i] = droot[i];
    dmi[i * n + i] = safe_invert(droot[i]);
  }
  std::vector<double> sym = matmul(dm, matmul(b, dm, n), n);
  for (int i = 0; i < n; i++)  // symmetrise away rounding before the eigensolve
    for (int j = i + 1; j < n; j++) {
      double m = 0.5 * (sym[i * n + j] + sym[j * n + i]);
      sym[i * n + j] = sym[j * n + i] = m;
    }
  Diagd dd;
  dd.n = n;
  std::vector<double> u;
  jacobi_eigen(sym, n, dd.l, u);
  dd.x = matmul(dmi, u, n);
  dd.xit = matmul(dm, u, n);
  return dd;
}

// b_ii = -(1/pi_i) sum_{k != i} r_ki pi_k              (diagd.ml:140-152)
static std::vector<double> b_of_exchangeable_pair(const std::vector<double> &r, const std::vector<double> &pi,
                                                  int n) {
  std::vector<double> b((size_t)n * n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      if (i != j) b[i * n + j] = r[i * n + j];
      else {
        double total = 0;
        for (int k = 0; k < n; k++)
          if (k != i) total += r[k * n + i] * pi[k];
        b[i * n + j] = -(total * safe_invert(pi[i]));
      }
    }
  return b;
}

// normed_of_exchangeable_pair: scale lambda so the mean rate is one (diagd.ml:156-172)
static Diagd normed_of_exchangeable_pair(const std::vector<double> &r, const std::vector<double> &pi, int n) {
  Diagd dd = of_d_b(pi, b_of_exchangeable_pair(r, pi, n), n);
  std::vector<double> q((size_t)n * n);
  dediagonalize(q.data(), dd.x.data(), dd.l.data(), dd.xit.data(), n);
  double rate = 0;
  for (int i = 0; i < n; i++) rate = rate - q[i * n + i] * pi[i];
  double f = 1. / rate;
  for (int i = 0; i < n; i++) dd.l[i] *= f;
  return dd;
}

// multi_exp: dst[r] = X diag(exp(rate_r * bl * l)) X^-1 (diagd.ml:79-98)
static void multi_exp(std::vector<double> &dst, const Diagd &dd, const std::vector<double> &rates, double bl,
                      const std::vector<char> *mask) {
  int n = dd.n;
  dst.assign(rates.size() * n * n, 0.0);
  std::vector<double> util(n);
  for (size_t r = 0; r < rates.size(); r++) {
    if (mask && !(*mask)[r]) continue;
    for (int i = 0; i < n; i++) util[i] = std::exp(rates[r] * bl * dd.l[i]);
    dediagonalize(&dst[r * n * n], dd.x.data(), util.data(), dd.xit.data(), n);
  }
}

// ---------------------------------------------------------------------------
// Discrete gamma rates (pplacer_src/gamma.ml:14-70, Yang 1994).
// ---------------------------------------------------------------------------
// Regularised lower incomplete gamma P(a, x): power series for x < a + 1,
// modified-Lentz continued fraction for Q = 1 - P otherwise.
static double gamma_p(double a, double x) {
  if (x <= 0) return 0.0;
  double lg = std::lgamma(a);
  if (x < a + 1) {
    double ap = a, sum = 1.0 / a, del = sum;
    for (int n = 0; n < 100000; n++) {
      ap += 1;
      del *= x / ap;
      sum += del;
      if (std::fabs(del) < std::fabs(sum) * 1e-17) break;
    }
    return sum * std::exp(-x + a * std::log(x) - lg);
  }
  double b = x + 1 - a, c = 1 / 1e-300, d = 1 / b, h = d;
  for (int i = 1; i < 100000; i++) {
    double an = -i * (i - a);
    b += 2;
    d = an * d + b;
    if (std::fabs(d) < 1e-300) d = 1e-300;
    c = b + an / c;
    if (std::fabs(c) < 1e-300) c = 1e-300;
    d = 1 / d;
    double del = d * c;
    h *= del;
    if (std::fabs(del - 1) < 1e-17) break;
  }
  return 1.0 - std::exp(-x + a * std::log(x) - lg) * h;
}

// Inverse of P(a, .): bracket then safeguarded Newton to full precision.
static double gamma_p_inv(double a, double p) {
  double lo = 0, hi = std::max(1.0, a);
  while (gamma_p(a, hi) < p) hi *= 2;
  double x = 0.5 * (lo + hi), lg = std::lgamma(a);
  for (int it = 0; it < 500; it++) {
    double f = gamma_p(a, x) - p;
    if (f < 0) lo = x; else hi = x;
    double dens = std::exp((a - 1) * std::log(x) - x - lg);
    double xn = (dens > 0) ? x - f / dens : 0.5 * (lo + hi);
    if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
    if (std::fabs(xn - x) <= 1e-16 * std::fabs(x) || hi - lo <= 1e-16 * hi) { x = xn; break; }
    x = xn;
  }
  return x;
}

// discrete_gamma n_cat alpha: category means, normalised to mean 1 (gamma.ml:52-70)
static std::vector<double> discrete_gamma(int n_cat, double alpha) {
  std::vector<double> freq(n_cat + 1);
  for (int i = 0; i <= n_cat; i++) {
    if (i == 0) freq[i] = 0.;
    else if (i == n_cat) freq[i] = 1.;
    else {
      double y = (double)i / (double)n_cat;
      // inverse_gamma_cdf ~alpha ~beta:1 with epsilon 1e-7 (gamma.ml:14-25)
      double cut = (y < gamma_p(alpha, 1e-7)) ? 0. : gamma_p_inv(alpha, y);
      freq[i] = gamma_p(alpha + 1., cut);
    }
  }
  std::vector<double> v(n_cat);
  double tot = 0;
  for (int i = 0; i < n_cat; i++) { v[i] = freq[i + 1] - freq[i]; tot += v[i]; }
  for (int i = 0; i < n_cat; i++) v[i] = (double)n_cat * v[i] / tot;  // make_mean_one, gamma.ml:27-30
  return v;
}

// ---------------------------------------------------------------------------
// Character -> likelihood vector (pplacer_src/nuc_models.ml:24-45,
// pplacer_src/prot_models.ml:5-43); informative = not '-' or '?'
// (common_src/alignment.ml:235).
// ---------------------------------------------------------------------------
static const char *kNucCodes = "ACGTRYMKSWHBVDN-?X";
static const int kNucBits[18] = {1, 2, 4, 8, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 15, 15, 15};
static const char *kProtCodes = "ARNDCQEGHILKMFPSTWYV";

static bool lv_of_char(char c, int K, double *lv) {
  if (K == 4) {
    const char *p = std::strchr(kNucCodes, c);
    if (!p || c == 0) return false;
    int bits = kNucBits[p - kNucCodes];
    for (int k = 0; k < 4; k++) lv[k] = (bits >> k) & 1 ? 1. : 0.;
    return true;
  }
  for (int k = 0; k < K; k++) lv[k] = 0.;
  if (c == '-' || c == '?' || c == 'X') { for (int k = 0; k < K; k++) lv[k] = 1.; return true; }
  auto idx = [](char ch) { const char *p = std::strchr(kProtCodes, ch); return (int)(p - kProtCodes); };
  if (c == 'B') { lv[idx('D')] = 1; lv[idx('N')] = 1; return true; }
  if (c == 'J') { lv[idx('I')] = 1; lv[idx('L')] = 1; return true; }
  if (c == 'Z') { lv[idx('E')] = 1; lv[idx('Q')] = 1; return true; }
  const char *p = std::strchr(kProtCodes, c);
  if (!p || c == 0) return false;
  lv[p - kProtCodes] = 1.;
  return true;
}
static inline bool informative(char c) { return c != '-' && c != '?'; }

// ---------------------------------------------------------------------------
// Models and GLVs (pplacer_src/gmix_model.ml, pplacer_src/gcat_model.ml)
// ---------------------------------------------------------------------------
struct Model {
  int K = 4;
  bool gcat = false;
  std::vector<double> statd, rates;  // rates: Gamma category rates or CAT rates
  Diagd dd;
  std::vector<int> site_cats;        // Gcat only, per (pre-masked) site
  std::vector<char> occupied;        // Gcat only
  int R() const { return gcat ? 1 : (int)rates.size(); }  // GLV planes
};

struct Glv {
  int R = 0, S = 0, K = 0;
  std::vector<double> a;  // [R][S][K]
  std::vector<int> e;     // [S]
  void make(int r, int s, int k) { R = r; S = s; K = k; a.assign((size_t)r * s * k, 0.0); e.assign(s, 0); }
  double *plane(int r) { return a.data() + (size_t)r * S * K; }
  const double *plane(int r) const { return a.data() + (size_t)r * S * K; }
};

static const double kLog2 = std::log(2.);

static double total_twoexp(const std::vector<int> &e) {  // gstar_support.ml:43-49
  double t = 0;
  for (int v : e) t += (double)v;
  return t;
}

// evolve_into: dst.e = src.e; dst = P(bl) src per rate (gmix_model.ml:308-315)
// or per site category (gcat_model.ml:327-345).  reind: masked site -> site.
static void evolve_into(const Model &m, Glv &dst, const Glv &src, double bl, const std::vector<int> *reind,
                        std::vector<double> &tensor) {
  int K = m.K;
  dst.e = src.e;
  if (!m.gcat) {
    multi_exp(tensor, m.dd, m.rates, bl, nullptr);
    for (int r = 0; r < src.R; r++) gemmish(dst.plane(r), &tensor[(size_t)r * K * K], src.plane(r), src.S, K);
    return;
  }
  std::vector<char> mask(m.rates.size(), 0);
  if (reind) for (int i : *reind) mask[m.site_cats[i]] = 1;
  else mask = m.occupied;
  multi_exp(tensor, m.dd, m.rates, bl, &mask);
  for (int i = 0; i < src.S; i++) {
    int cat = m.site_cats[reind ? (*reind)[i] : i];
    const double *P = &tensor[(size_t)cat * K * K];
    const double *v = &src.a[(size_t)i * K];
    double *y = &dst.a[(size_t)i * K];
    for (int r = 0; r < K; r++) {  // gemv, alpha 1, beta 0
      double t = 0;
      for (int j = 0; j < K; j++) t += P[r * K + j] * v[j];
      y[r] = t;
    }
  }
}

static void glv_pairwise_prod(Glv &dst, const Glv &x, const Glv &y) {  // gmix_model.ml:215-218
  for (int s = 0; s < x.S; s++) dst.e[s] = x.e[s] + y.e[s];
  pairwise_prod(dst.a.data(), x.a.data(), y.a.data(), x.a.size());
}

static void listwise_prod(Glv &dst, const std::vector<const Glv *> &l) {  // gmix_model.ml:224-233
  if (l.size() == 1) { dst.e = l[0]->e; dst.a = l[0]->a; return; }
  glv_pairwise_prod(dst, *l[0], *l[1]);
  for (size_t i = 2; i < l.size(); i++) glv_pairwise_prod(dst, dst, *l[i]);
}

static void statd_pairwise_prod_glv(const Model &m, Glv &dst, const Glv &g1, const Glv &g2) {
  for (int s = 0; s < g1.S; s++) dst.e[s] = g1.e[s] + g2.e[s];  // gmix_model.ml:319-322
  statd_pairwise_prod(m.statd.data(), dst.a.data(), g1.a.data(), g2.a.data(), (size_t)g1.R * g1.S, g1.K);
}

// perhaps_pull_exponent (gmix_model.ml:163-187, gcat_model.ml:195-212)
static void perhaps_pull_exponent(int min_allowed_twoexp, Glv &g) {
  for (int s = 0; s < g.S; s++) {
    int max_twoexp = -(int)0x3fffffff;
    for (int r = 0; r < g.R; r++) {
      const double *v = g.plane(r) + (size_t)s * g.K;
      double mx = v[0];
      for (int k = 1; k < g.K; k++) mx = std::max(mx, v[k]);
      int te;
      std::frexp(mx, &te);
      if (te > max_twoexp) max_twoexp = te;
    }
    if (max_twoexp < min_allowed_twoexp) {
      double f = std::ldexp(0.5, -max_twoexp + 1);  // of_twoexp, gstar_support.ml:40
      for (int r = 0; r < g.R; r++) {
        double *v = g.plane(r) + (size_t)s * g.K;
        for (int k = 0; k < g.K; k++) v[k] *= f;
      }
      g.e[s] += max_twoexp;
    }
  }
}

// log_like3 (gmix_model.ml:298-304, gcat_model.ml:317-323)
static double log_like3(const Model &m, std::vector<double> &util, const Glv &x, const Glv &y, const Glv &z) {
  double core = m.gcat ? mat_log_like3(m.statd.data(), x.a.data(), y.a.data(), z.a.data(), x.S, x.K)
                       : ten_log_like3(m.statd.data(), x.a.data(), y.a.data(), z.a.data(), util.data(), x.R,
                                       x.S, x.K);
  return core + kLog2 * ((total_twoexp(x.e) + total_twoexp(y.e)) + total_twoexp(z.e));
}

// masked_logdot (gmix_model.ml:194-198, gcat_model.ml:220-224)
static double masked_logdot(const Model &m, std::vector<double> &util, const Glv &x, const Glv &y,
                            const std::vector<uint16_t> &mask) {
  double core = m.gcat ? mat_masked_logdot(x.a.data(), y.a.data(), mask.data(), x.S, x.K)
                       : ten_masked_logdot(x.a.data(), y.a.data(), mask.data(), util.data(), x.R, x.S, x.K);
  double ex = 0, ey = 0;
  for (int s = 0; s < x.S; s++) if (mask[s]) ex += (double)x.e[s];
  for (int s = 0; s < y.S; s++) if (mask[s]) ey += (double)y.e[s];
  return core + kLog2 * (ex + ey);
}

// logdot = bounded_logdot over all sites (gmix_model.ml:202-212, gcat_model.ml:230-239)
static double logdot(const Model &m, std::vector<double> &util, const Glv &x, const Glv &y) {
  int last = x.S - 1;
  double core = m.gcat ? mat_bounded_logdot(x.a.data(), y.a.data(), 0, last, x.K)
                       : ten_bounded_logdot(x.a.data(), y.a.data(), 0, last, util.data(), x.R, x.S, x.K);
  return core + kLog2 * (total_twoexp(x.e) + total_twoexp(y.e));
}

// slow_log_like3: per-site sum with 1/R inside the log (gmix_model.ml:325-351,
// gcat_model.ml:355-378); throws on a zero-likelihood site.
static double slow_log_like3(const Model &m, const Glv &x, const Glv &y, const Glv &z) {
  double tot = 0;
  double fr = (double)x.R;
  for (int s = 0; s < x.S; s++) {
    double sl = 0;
    for (int r = 0; r < x.R; r++)
      for (int k = 0; k < x.K; k++) {
        size_t i = ((size_t)r * x.S + s) * x.K + k;
        sl = sl + m.statd[k] * x.a[i] * y.a[i] * z.a[i];
      }
    if (0. >= sl) throw std::runtime_error("zero site likelihood");
    double v = m.gcat ? std::log(sl) : std::log(sl / fr);
    tot += v + kLog2 * (double)(x.e[s] + y.e[s] + z.e[s]);
  }
  return tot;
}

// ---------------------------------------------------------------------------
// Reference tree: darr / parr / snodes (pplacer_src/like_stree.ml:43-110,
// pplacer_src/pplacer_run.ml:322-340, pplacer_src/glv_arr.ml:46-57).
// Nodes are numbered post-order (newick_parser.mly:50-59); children of a node
// in increasing id order reproduce the Newick child order.
// ---------------------------------------------------------------------------
struct Ref {
  const Model *m = nullptr;
  int n_nodes = 0, root = -1, S = 0;
  std::vector<int> parent;
  std::vector<double> bl;
  std::vector<std::vector<int>> children;
  std::vector<Glv> darr, parr, snodes;
};

static void build_reference(Ref &ref, const Model &m, int n_nodes, const int *parent, const double *bl, int S,
                            const int *leaf_row, const char *leaf_seqs) {
  ref.m = &m;
  ref.n_nodes = n_nodes;
  ref.S = S;
  ref.parent.assign(parent, parent + n_nodes);
  ref.bl.assign(bl, bl + n_nodes);
  ref.children.assign(n_nodes, {});
  for (int i = 0; i < n_nodes; i++) {
    if (parent[i] < 0) ref.root = i;
    else ref.children[parent[i]].push_back(i);
  }
  ref.bl[ref.root] = 0.;  // add_zero_root_bl (newick_gtree.ml:145-157)
  int R = m.R(), K = m.K;
  std::vector<Glv> distal(n_nodes), evd(n_nodes), prox(n_nodes);
  std::vector<double> tensor;
  std::vector<double> lv(K);
  // post-order: ids are already post-order so increasing id visits children first
  for (int id = 0; id < n_nodes; id++) {
    Glv &d = distal[id];
    d.make(R, S, K);
    if (ref.children[id].empty()) {  // prep_constant_rate_glv_from_lv_arr (gmix_model.ml:149-156)
      const char *seq = leaf_seqs + (size_t)leaf_row[id] * S;
      for (int s = 0; s < S; s++) {
        if (!lv_of_char(seq[s], K, lv.data())) throw std::runtime_error("unknown character in reference");
        for (int r = 0; r < R; r++)
          for (int k = 0; k < K; k++) d.a[((size_t)r * S + s) * K + k] = lv[k];
      }
    } else {
      std::vector<const Glv *> l;
      for (int c : ref.children[id]) l.push_back(&evd[c]);
      listwise_prod(d, l);
      perhaps_pull_exponent(-50, d);  // like_stree.ml:8,56-61
    }
    evd[id].make(R, S, K);
    evolve_into(m, evd[id], d, ref.bl[id], nullptr, tensor);
  }
  // pre-order proximal (like_stree.ml:74-100)
  for (int i = 0; i < n_nodes; i++) prox[i].make(R, S, K);
  std::fill(prox[ref.root].a.begin(), prox[ref.root].a.end(), 1.0);  // set_unit
  std::vector<int> stack = {ref.root};
  Glv evolved_prox;
  evolved_prox.make(R, S, K);
  std::vector<int> order;
  while (!stack.empty()) {  // pre-order: parent before children
    int id = stack.back();
    stack.pop_back();
    order.push_back(id);
    for (auto it = ref.children[id].rbegin(); it != ref.children[id].rend(); ++it) stack.push_back(*it);
  }
  for (int id : order) {
    if (ref.children[id].empty()) continue;
    evolve_into(m, evolved_prox, prox[id], ref.bl[id], nullptr, tensor);
    for (int chosen : ref.children[id]) {
      std::vector<const Glv *> l = {&evolved_prox};
      for (int c : ref.children[id])
        if (c != chosen) l.push_back(&evd[c]);
      listwise_prod(prox[chosen], l);
      perhaps_pull_exponent(-50, prox[chosen]);
    }
  }
  // pull exponents at -10 and build supernodes (pplacer_run.ml:332-340)
  for (int i = 0; i < n_nodes; i++) {
    perhaps_pull_exponent(-10, distal[i]);
    perhaps_pull_exponent(-10, prox[i]);
  }
  ref.snodes.resize(n_nodes);
  Glv ud, up;
  ud.make(R, S, K);
  up.make(R, S, K);
  for (int i = 0; i < n_nodes; i++) {
    ref.snodes[i].make(R, S, K);
    evolve_into(m, ud, distal[i], ref.bl[i] / 2., nullptr, tensor);
    evolve_into(m, up, prox[i], ref.bl[i] / 2., nullptr, tensor);
    statd_pairwise_prod_glv(m, ref.snodes[i], ud, up);
  }
  ref.darr = std::move(distal);
  ref.parr = std::move(prox);
}

// ---------------------------------------------------------------------------
// Brent minimisation with GSL's conventions (pplacer_src/minimization.ml:24-41,
// 83-101 calling gsl_min_fminimizer_brent).
// ---------------------------------------------------------------------------
struct GslError {};          // Gsl.Error.Gsl_exn
struct ExceededMaxIter {};   // Minimization.ExceededMaxIter
struct StartFailure {};      // InvalidStartValues / FindStartFailure
struct FoundMin { double x; };

template <class F>
static double gsl_checked(F &f, double x) {  // SAFE_FUNC_CALL: non-finite values are errors
  double v = f(x);
  if (!std::isfinite(v)) throw GslError{};
  return v;
}

template <class F>
static double bisection_start_finder(F &f, double raw_start, double left, double right, double tol,
                                     int max_iters) {
  if (left >= raw_start || raw_start >= right) throw StartFailure{};
  double righty = f(right);  // OCaml evaluates the tuple (f left, f right) right to left
  double lefty = f(left);
  double smaller = lefty < righty ? left : right;
  double miny = lefty <= righty ? lefty : righty;  // Stdlib.min
  double prev = raw_start;
  for (int iter = 1;; iter++) {
    double pv = f(prev);
    if (pv < miny) return prev;
    if (std::fabs(prev - smaller) < tol) throw FoundMin{pv < miny ? prev : smaller};
    if (iter > max_iters) throw StartFailure{};
    prev = (prev + smaller) / 2.;
  }
}

template <class F>
static double brent(F &f, double raw_start, double left, double right, double tol, int max_iters = 100) {
  double start;
  try {
    start = bisection_start_finder(f, raw_start, left, right, tol, max_iters);
  } catch (FoundMin &fm) {
    return fm.x;
  }
  // gsl_min_fminimizer_set: f at lower, upper, minimum; bracket checks
  double xl = left, xu = right, xm = start;
  double fl = gsl_checked(f, xl), fu = gsl_checked(f, xu), fm = gsl_checked(f, xm);
  if (xl > xu || xm >= xu || xm <= xl || fm >= fl || fm >= fu) throw GslError{};
  const double golden = 0.3819660;  // (3 - sqrt 5) / 2 to 7 digits, as GSL
  double v = xl + golden * (xu - xl), w = v;
  double fv = gsl_checked(f, v), fw = fv;
  double d = 0, e = 0;
  for (int step = 1;; step++) {
    if (step > max_iters) throw ExceededMaxIter{};
    // one Brent iteration (parabolic step, else golden section)
    double z = xm, fz = fm;
    double dd = e, ee = d;  // GSL swaps the roles of d and e on entry
    double wl = z - xl, wu = xu - z;
    double tolerance = 1.4901161193847656e-08 * std::fabs(z);  // sqrt(DBL_EPSILON) |z|
    double p = 0, q = 0, r = 0;
    double mid = 0.5 * (xl + xu);
    double u;
    if (std::fabs(ee) > tolerance) {
      r = (z - w) * (fz - fv);
      q = (z - v) * (fz - fw);
      p = (z - v) * q - (z - w) * r;
      q = 2 * (q - r);
      if (q > 0) p = -p; else q = -q;
      r = ee;
      ee = dd;
    }
    if (std::fabs(p) < std::fabs(0.5 * q * r) && p < q * wl && p < q * wu) {
      double t2 = 2 * tolerance;
      dd = p / q;
      u = z + dd;
      if ((u - xl) < t2 || (xu - u) < t2) dd = (z < mid) ? tolerance : -tolerance;
    } else {
      ee = (z < mid) ? xu - z : -(z - xl);
      dd = golden * ee;
    }
    if (std::fabs(dd) >= tolerance) u = z + dd;
    else u = z + ((dd > 0) ? tolerance : -tolerance);
    e = ee;
    d = dd;
    double fuv = gsl_checked(f, u);
    if (fuv <= fz) {
      if (u < z) { xu = z; fu = fz; } else { xl = z; fl = fz; }
      v = w; fv = fw; w = z; fw = fz;
      xm = u; fm = fuv;
    } else {
      if (u < z) { xl = u; fl = fuv; } else { xu = u; fu = fuv; }
      if (fuv <= fw || w == z) { v = w; fv = fw; w = u; fw = fuv; }
      else if (fuv <= fv || v == z || v == w) { v = u; fv = fuv; }
    }
    if (xu - xl < tol) return xm;
  }
}

// ---------------------------------------------------------------------------
// Placement core (pplacer_src/core.ml:113-409, three_tax.ml:15-85,
// glv_edge.ml:29-44).
// ---------------------------------------------------------------------------
struct Prefs {
  double start_pend = 0.1, max_pend = 2., initial_tolerance = 0.01;
  int max_strikes = 6;
  double strike_box = 3.;
  int max_pitches = 40, keep_at_most = 7;
  double keep_factor = 0.01;
};

struct Placement {
  int edge;
  double like, lwr, dist, pend;
};

struct QueryOut {
  int status = 0;  // 0 ok, 1 no informative sites, 2 empty results, 3 unknown char, 4 start failure
  std::vector<Placement> pl;
  std::vector<std::pair<int, double>> ranking;  // stage-1 order (edge, score)
  std::vector<std::pair<int, double>> stage2;   // edges tried in stage 2 with their like
};

struct GlvEdge {  // glv_edge.ml
  Glv orig, evolv;
  double bl = 0;
};

struct Placer {
  const Ref &ref;
  const Model &m;
  Prefs prefs;
  std::vector<double> util, tensor;
  int trial_loc = -1;
  double trial_pend = 0, trial_dist = 0, trial_tol = 0;
  Placer(const Ref &r, const Prefs &p) : ref(r), m(*r.m), prefs(p) { util.assign(r.S + 1, 0.); }

  void set_bl(GlvEdge &ge, double bl, const std::vector<int> *reind) {
    ge.bl = bl;
    evolve_into(m, ge.evolv, ge.orig, bl, reind, tensor);
  }

  // FP64 logL and its derivatives at (pend, dist) for location loc
  // (the CPU reference for the GPU adjoint): out = L, dL/dp, dL/dd,
  // d2L/dp2, d2L/dd2, d2L/dp dd with prox = bl(loc) - dist.
  int derivs(const char *seq, int loc, double pend, double dist, double *out) {
    int S = ref.S, K = m.K, R = m.R();
    std::vector<int> reind;
    std::vector<double> lv(K);
    for (int s = 0; s < S; s++) {
      if (!lv_of_char(seq[s], K, lv.data())) return 3;
      if (informative(seq[s])) reind.push_back(s);
    }
    if (reind.empty()) return 1;
    int NM = (int)m.rates.size();
    double cut = ref.bl[loc], prox = cut - dist;
    // P, P', P'' for each matrix index at t in {dist, prox, pend}
    auto pm = [&](double t, int deriv, std::vector<double> &out_m) {
      out_m.assign((size_t)NM * K * K, 0.0);
      for (int mm = 0; mm < NM; mm++)
        for (int i = 0; i < K; i++)
          for (int j = 0; j < K; j++) {
            double acc = 0;
            for (int k = 0; k < K; k++) {
              double lr = m.rates[mm] * m.dd.l[k];
              double f = std::exp(lr * t) * (deriv == 0 ? 1.0 : deriv == 1 ? lr : lr * lr);
              acc += f * m.dd.x[i * K + k] * m.dd.xit[j * K + k];
            }
            out_m[((size_t)mm * K + i) * K + j] = acc;
          }
    };
    std::vector<double> Pd[3], Pp[3], Pz[3];
    for (int dv = 0; dv < 3; dv++) { pm(dist, dv, Pd[dv]); pm(prox, dv, Pp[dv]); pm(pend, dv, Pz[dv]); }
    double L = 0, gp = 0, gd = 0, hpp = 0, hdd = 0, hpd = 0;
    long long esum = 0;
    for (int i : reind) {
      lv_of_char(seq[i], K, lv.data());
      esum += (long long)ref.darr[loc].e[i] + ref.parr[loc].e[i];
      double u = 0, ud = 0, udd = 0, up = 0, upp = 0, upd = 0;
      for (int r = 0; r < R; r++) {
        int mm = m.gcat ? m.site_cats[i] : r;
        const double *D = &ref.darr[loc].a[((size_t)r * S + i) * K];
        const double *Pr = &ref.parr[loc].a[((size_t)r * S + i) * K];
        for (int k = 0; k < K; k++) {
          double x[3] = {0, 0, 0}, y[3] = {0, 0, 0}, z[3] = {0, 0, 0};
          for (int dv = 0; dv < 3; dv++)
            for (int j = 0; j < K; j++) {
              size_t o = ((size_t)mm * K + k) * K + j;
              x[dv] += Pd[dv][o] * D[j];
              y[dv] += Pp[dv][o] * Pr[j];
              z[dv] += Pz[dv][o] * lv[j];
            }
          double pi = m.statd[k];
          double xy = x[0] * y[0], a = x[1] * y[0] - x[0] * y[1];
          double b = x[2] * y[0] - 2 * x[1] * y[1] + x[0] * y[2];
          u += pi * z[0] * xy;
          ud += pi * z[0] * a;
          udd += pi * z[0] * b;
          up += pi * z[1] * xy;
          upp += pi * z[2] * xy;
          upd += pi * z[1] * a;
        }
      }
      L += std::log(u);
      double lp = up / u, ld = ud / u;
      gp += lp; gd += ld;
      hpp += upp / u - lp * lp;
      hdd += udd / u - ld * ld;
      hpd += upd / u - lp * ld;
    }
    if (!m.gcat) L -= ((float)reind.size()) * std::log((double)(float)R);
    L += kLog2 * (double)esum;
    out[0] = L; out[1] = gp; out[2] = gd; out[3] = hpp; out[4] = hdd; out[5] = hpd;
    return 0;
  }

  QueryOut process(const char *seq, bool keep_trace) {
    QueryOut out;
    int S = ref.S, K = m.K, R = m.R();
    std::vector<double> lv(K);
    // full-length query GLV evolved by start_pend (core.ml:107-141)
    Glv fq, fqe;
    fq.make(R, S, K);
    fqe.make(R, S, K);
    std::vector<char> mask_arr(S);
    std::vector<uint16_t> mask_vec(S);
    std::vector<int> reind;
    for (int s = 0; s < S; s++) {
      if (!lv_of_char(seq[s], K, lv.data())) { out.status = 3; return out; }
      for (int r = 0; r < R; r++)
        for (int k = 0; k < K; k++) fq.a[((size_t)r * S + s) * K + k] = lv[k];
      mask_arr[s] = informative(seq[s]);
      mask_vec[s] = mask_arr[s] ? 1 : 0;
      if (mask_arr[s]) reind.push_back(s);
    }
    evolve_into(m, fqe, fq, prefs.start_pend, nullptr, tensor);
    int Sq = (int)reind.size();
    if (Sq == 0) { out.status = 1; return out; }
    const std::vector<int> *rp = m.gcat ? &reind : nullptr;  // core.ml:175-179
    GlvEdge pend, dist, prox;
    pend.orig.make(R, Sq, K);
    for (int i = 0; i < Sq; i++) {
      lv_of_char(seq[reind[i]], K, lv.data());
      for (int r = 0; r < R; r++)
        for (int k = 0; k < K; k++) pend.orig.a[((size_t)r * Sq + i) * K + k] = lv[k];
    }
    pend.evolv = pend.orig;
    dist.orig.make(R, Sq, K);
    dist.evolv = dist.orig;
    prox.orig = dist.orig;
    prox.evolv = dist.orig;
    set_bl(pend, prefs.start_pend, rp);
    // stage 1: rank every non-root edge (core.ml:187-197, fig.ml:101-105,143-147)
    std::vector<std::pair<double, int>> scored;
    for (int loc = 0; loc < ref.n_nodes; loc++) {
      if (loc == ref.root) continue;
      scored.push_back({masked_logdot(m, util, fqe, ref.snodes[loc], mask_vec), loc});
    }
    std::stable_sort(scored.begin(), scored.end(),
                     [](const std::pair<double, int> &a, const std::pair<double, int> &b) { return a.first > b.first; });
    if (keep_trace)
      for (auto &p : scored) out.ranking.push_back({p.second, p.first});

    auto mask_into = [&](const Glv &src, Glv &dst) {  // gmix_model.ml:130-141
      for (int i = 0; i < Sq; i++) {
        dst.e[i] = src.e[reind[i]];
        for (int r = 0; r < R; r++)
          std::memcpy(&dst.a[((size_t)r * Sq + i) * K], &src.a[((size_t)r * S + reind[i]) * K], K * sizeof(double));
      }
    };
    auto set_tt_edges = [&](int loc, double pendant, double distal) {  // core.ml:225-239
      double cut = ref.bl[loc];
      set_bl(pend, pendant, rp);
      mask_into(ref.darr[loc], dist.orig);
      set_bl(dist, distal, rp);
      mask_into(ref.parr[loc], prox.orig);
      set_bl(prox, cut - distal, rp);
    };
    auto tt_default = [&](int loc) { set_tt_edges(loc, prefs.start_pend, ref.bl[loc] / 2.); };
    auto log_like = [&]() { return log_like3(m, util, prox.evolv, dist.evolv, pend.evolv); };  // three_tax.ml:30-36
    auto set_dist_bl = [&](double d) {  // three_tax.ml:41-45
      double prox_bl = (dist.bl + prox.bl) - d;
      set_bl(dist, d, rp);
      set_bl(prox, prox_bl, rp);
    };
    auto optimize_something = [&](double tol, int which, double start_v, double min_v, double max_v) {
      if (min_v == max_v) return start_v;  // three_tax.ml:48-58
      auto f = [&](double v) {
        if (which == 0) set_bl(pend, v, rp); else set_dist_bl(v);
        return -log_like();
      };
      return brent(f, start_v, min_v, max_v, tol);
    };
    auto optimize = [&](double tol) {  // three_tax.ml:70-83, core.ml:10
      double prev_pend = pend.bl, prev_dist = dist.bl;
      for (int step = 1;; step++) {
        if (step > 200) throw ExceededMaxIter{};
        double cp = optimize_something(tol, 0, pend.bl, 1e-8, prefs.max_pend);
        double cd = optimize_something(tol, 1, dist.bl, 0., dist.bl + prox.bl);
        if (std::fabs(prev_pend - cp) > tol || std::fabs(prev_dist - cd) > tol) { prev_pend = cp; prev_dist = cd; }
        else break;
      }
    };
    struct Res { double like, pend, dist; };
    auto ml_optimize_location = [&](double tol) {  // core.ml:255-271
      try { optimize(tol); } catch (ExceededMaxIter &) {}
      return Res{log_like(), pend.bl, dist.bl};
    };
    auto safe_ml_optimize_location = [&](double tol, int loc) {  // core.ml:272-279
      try { return ml_optimize_location(tol); }
      catch (GslError &) { tt_default(loc); return ml_optimize_location(tol); }
    };

    if (trial_loc >= 0) {  // one location from a given start (core.ml:255-279 after set_tt_edges)
      set_tt_edges(trial_loc, trial_pend, trial_dist);
      try {
        Res r = safe_ml_optimize_location(trial_tol, trial_loc);
        out.pl.push_back({trial_loc, r.like, 1.0, r.dist, r.pend});
      } catch (GslError &) { out.status = 2; }
      catch (StartFailure &) { out.status = 4; }
      return out;
    }
    long t_max_pitches, t_max_strikes;  // core.ml:96-106
    if (prefs.max_strikes == 0) { t_max_pitches = 1L << 60; t_max_strikes = 1L << 60; }
    else { t_max_pitches = prefs.max_pitches; t_max_strikes = prefs.max_strikes; }
    // stage 2: baseball (core.ml:283-318)
    std::vector<std::pair<int, Res>> results;
    double like_record = -INFINITY;
    long n_strikes = 0;
    try {
      for (auto &sc : scored) {
        int loc = sc.second;
        tt_default(loc);
        Res r;
        try { r = safe_ml_optimize_location(prefs.initial_tolerance, loc); }
        catch (GslError &) { continue; }
        long before = (long)results.size();
        results.push_back({loc, r});
        if (keep_trace) out.stage2.push_back({loc, r.like});
        if (before >= t_max_pitches) break;
        if (r.like > like_record) like_record = r.like;
        else if (r.like < like_record - prefs.strike_box) {
          if (n_strikes + 1 >= t_max_strikes) break;
          n_strikes++;
        }
      }
    } catch (StartFailure &) { out.status = 4; return out; }
    if (results.empty()) { out.status = 2; return out; }
    // sort, keep, refine (core.ml:336-377)
    std::vector<std::pair<int, Res>> sorted = results;
    std::stable_sort(sorted.begin(), sorted.end(),
                     [](const std::pair<int, Res> &a, const std::pair<int, Res> &b) { return a.second.like > b.second.like; });
    double best = sorted[0].second.like;
    double log_keep = std::log(prefs.keep_factor);
    std::vector<std::pair<int, Res>> keep;
    for (size_t i = 0; i < sorted.size(); i++)
      if ((long)i < prefs.keep_at_most && sorted[i].second.like >= log_keep + best) keep.push_back(sorted[i]);
    std::vector<std::pair<int, Res>> refined;
    try {
      for (auto &kr : keep) {
        set_tt_edges(kr.first, kr.second.pend, kr.second.dist);
        try { refined.push_back({kr.first, safe_ml_optimize_location(1e-5, kr.first)}); }
        catch (GslError &) { refined.push_back(kr); }
      }
    } catch (StartFailure &) { out.status = 4; return out; }
    // like_weight_ratio (common_src/ppatteries.ml:175-183) then sort by it (pquery.ml:8-9,92)
    std::vector<double> lw(refined.size());
    for (size_t i = 0; i < refined.size(); i++) {
      double tot = 0;
      for (size_t j = 0; j < refined.size(); j++) tot += std::exp(refined[j].second.like - refined[i].second.like);
      lw[i] = 1. / tot;
    }
    for (size_t i = 0; i < refined.size(); i++)
      out.pl.push_back({refined[i].first, refined[i].second.like, lw[i], refined[i].second.dist, refined[i].second.pend});
    std::stable_sort(out.pl.begin(), out.pl.end(), [](const Placement &a, const Placement &b) { return a.lwr > b.lwr; });
    return out;
  }
};

}  // namespace orc

// ---------------------------------------------------------------------------
// C API used by oracle/oracle.py
// ---------------------------------------------------------------------------
using namespace orc;

extern "C" {

// Restated L0 kernels, exported for comparison with oracle/_ref.
void orc_gemmish(double *dst, const double *a, const double *b, int n_sites, int n_states) {
  gemmish(dst, a, b, n_sites, n_states);
}
void orc_dediagonalize(double *dst, const double *u, const double *l, const double *uit, int n) {
  dediagonalize(dst, u, l, uit, n);
}
double orc_mat_log_like3(const double *statd, const double *x, const double *y, const double *z, int S, int K) {
  return mat_log_like3(statd, x, y, z, S, K);
}
void orc_pairwise_prod(double *dst, const double *x, const double *y, long n) { pairwise_prod(dst, x, y, (size_t)n); }
void orc_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b, long rows, int K) {
  statd_pairwise_prod(statd, dst, a, b, (size_t)rows, K);
}
double orc_mat_masked_logdot(const double *x, const double *y, const uint16_t *mask, int S, int K) {
  return mat_masked_logdot(x, y, mask, S, K);
}
double orc_mat_bounded_logdot(const double *x, const double *y, int first, int last, int K) {
  return mat_bounded_logdot(x, y, first, last, K);
}
double orc_ten_log_like3(const double *statd, const double *x, const double *y, const double *z, double *util, int R,
                         int S, int K) {
  return ten_log_like3(statd, x, y, z, util, R, S, K);
}
double orc_ten_masked_logdot(const double *x, const double *y, const uint16_t *mask, double *util, int R, int S,
                             int K) {
  return ten_masked_logdot(x, y, mask, util, R, S, K);
}
double orc_ten_bounded_logdot(const double *x, const double *y, int first, int last, double *util, int R, int S,
                              int K) {
  return ten_bounded_logdot(x, y, first, last, util, R, S, K);
}

void orc_discrete_gamma(int n_cat, double alpha, double *out) {
  std::vector<double> v = discrete_gamma(n_cat, alpha);
  std::copy(v.begin(), v.end(), out);
}
double orc_gamma_p(double a, double x) { return gamma_p(a, x); }

// Diagd of (d, b) without normalisation (diagd.ml:123) and the normalised
// exchangeable-pair form (diagd.ml:169-172).
void orc_diagd_of_d_b(int n, const double *d, const double *b, double *x, double *l, double *xit) {
  Diagd dd = of_d_b(std::vector<double>(d, d + n), std::vector<double>(b, b + n * n), n);
  std::copy(dd.x.begin(), dd.x.end(), x);
  std::copy(dd.l.begin(), dd.l.end(), l);
  std::copy(dd.xit.begin(), dd.xit.end(), xit);
}
void orc_diagd_normed(int n, const double *exch, const double *statd, double *x, double *l, double *xit) {
  Diagd dd = normed_of_exchangeable_pair(std::vector<double>(exch, exch + n * n), std::vector<double>(statd, statd + n), n);
  std::copy(dd.x.begin(), dd.x.end(), x);
  std::copy(dd.l.begin(), dd.l.end(), l);
  std::copy(dd.xit.begin(), dd.xit.end(), xit);
}
// to_exp (diagd.ml:65-71)
void orc_diagd_to_exp(int n, const double *x, const double *l, const double *xit, double bl, double *dst) {
  std::vector<double> u(n);
  for (int i = 0; i < n; i++) u[i] = std::exp(bl * l[i]);
  dediagonalize(dst, x, u.data(), xit, n);
}

// Model: exchangeabilities (n x n, symmetric, diagonal ignored), statd,
// rates; site_cats (n_site_cats entries) selects the per-site CAT model.
void *orc_model_new(int K, const double *exch, const double *statd, int n_rates, const double *rates,
                    int n_site_cats, const int *site_cats) {
  Model *m = new Model();
  m->K = K;
  m->statd.assign(statd, statd + K);
  m->rates.assign(rates, rates + n_rates);
  m->dd = normed_of_exchangeable_pair(std::vector<double>(exch, exch + K * K), m->statd, K);
  if (n_site_cats > 0) {
    m->gcat = true;
    m->site_cats.assign(site_cats, site_cats + n_site_cats);
    m->occupied.assign(n_rates, 0);
    for (int c : m->site_cats) m->occupied[c] = 1;  // gcat_model.ml:48-50
  }
  return m;
}
void orc_model_diagd(void *mp, double *x, double *l, double *xit) {
  Model *m = (Model *)mp;
  std::copy(m->dd.x.begin(), m->dd.x.end(), x);
  std::copy(m->dd.l.begin(), m->dd.l.end(), l);
  std::copy(m->dd.xit.begin(), m->dd.xit.end(), xit);
}
void orc_model_free(void *m) { delete (Model *)m; }

// Evolve a GLV ([R][S][K] with exponents) by bl (reind may be null).
void orc_evolve(void *mp, const double *src_a, const int *src_e, int S, double bl, const int *reind, double *dst_a,
                int *dst_e) {
  Model *m = (Model *)mp;
  Glv src, dst;
  src.make(m->R(), S, m->K);
  dst.make(m->R(), S, m->K);
  std::copy(src_a, src_a + src.a.size(), src.a.begin());
  std::copy(src_e, src_e + S, src.e.begin());
  std::vector<int> rv;
  if (reind) rv.assign(reind, reind + S);
  std::vector<double> tensor;
  evolve_into(*m, dst, src, bl, reind ? &rv : nullptr, tensor);
  std::copy(dst.a.begin(), dst.a.end(), dst_a);
  std::copy(dst.e.begin(), dst.e.end(), dst_e);
}

int orc_ref_new(void *mp, int n_nodes, const int *parent, const double *bl, int S, const int *leaf_row,
                const char *leaf_seqs, void **out) {
  Ref *r = new Ref();
  try {
    build_reference(*r, *(Model *)mp, n_nodes, parent, bl, S, leaf_row, leaf_seqs);
  } catch (std::exception &ex) {
    fprintf(stderr, "oracle: %s\n", ex.what());
    delete r;
    return 1;
  }
  *out = r;
  return 0;
}
void orc_ref_free(void *r) { delete (Ref *)r; }
// which: 0 darr, 1 parr, 2 snodes
void orc_ref_glv(void *rp, int which, int node, double *a, int *e) {
  Ref *r = (Ref *)rp;
  const Glv &g = which == 0 ? r->darr[node] : which == 1 ? r->parr[node] : r->snodes[node];
  std::copy(g.a.begin(), g.a.end(), a);
  std::copy(g.e.begin(), g.e.end(), e);
}
// Per-site log likelihood of the whole tree at the root, from the root's
// distal GLV (the product of its children's evolved GLVs): the values of
// Like_stree.site_log_like_arr (like_stree.ml:113-131) for a one-plane model.
void orc_ref_root_site_loglike(void *rp, double *out) {
  Ref *r = (Ref *)rp;
  const Model &m = *r->m;
  const Glv &g = r->darr[r->root];
  for (int s = 0; s < r->S; s++) {
    double u = 0;
    for (int k = 0; k < m.K; k++) u += m.statd[k] * g.a[(size_t)s * m.K + k];
    out[s] = std::log(u) + kLog2 * g.e[s];
  }
}

// Tree log likelihood seen from edge `node` (tests/pplacer/test_like.ml:57-66):
// out[0] = slow_log_like3(P(bl/2) d, P(bl/2) p, 1); out[1] = logdot(snode, 1).
void orc_ref_edge_loglike(void *rp, int node, double *out) {
  Ref *r = (Ref *)rp;
  const Model &m = *r->m;
  Glv ud, up, one;
  ud.make(m.R(), r->S, m.K);
  up.make(m.R(), r->S, m.K);
  one.make(m.R(), r->S, m.K);
  std::fill(one.a.begin(), one.a.end(), 1.0);
  std::vector<double> tensor, util(r->S);
  evolve_into(m, ud, r->darr[node], r->bl[node] / 2., nullptr, tensor);
  evolve_into(m, up, r->parr[node], r->bl[node] / 2., nullptr, tensor);
  out[0] = slow_log_like3(m, ud, up, one);
  out[1] = logdot(m, util, r->snodes[node], one);
}

struct OrcPrefs {
  double start_pend, max_pend, initial_tolerance;
  int max_strikes;
  double strike_box;
  int max_pitches, keep_at_most;
  double keep_factor;
};
struct OrcPlacement {
  int edge;
  int pad;
  double like, lwr, dist, pend;
};

// Place n_queries (each S chars, pre-masked alignment columns).  out has
// keep_at_most slots per query; n_out[q] = placements written, status[q] as
// QueryOut::status.  Work is split over n_threads host threads.
void orc_place(void *rp, const OrcPrefs *pp, int n_queries, const char *seqs, int n_threads, OrcPlacement *out,
               int *n_out, int *status) {
  Ref *r = (Ref *)rp;
  Prefs p;
  p.start_pend = pp->start_pend; p.max_pend = pp->max_pend; p.initial_tolerance = pp->initial_tolerance;
  p.max_strikes = pp->max_strikes; p.strike_box = pp->strike_box; p.max_pitches = pp->max_pitches;
  p.keep_at_most = pp->keep_at_most; p.keep_factor = pp->keep_factor;
  std::atomic<int> next(0);
  auto worker = [&]() {
    Placer pl(*r, p);
    for (;;) {
      int q = next.fetch_add(1);
      if (q >= n_queries) break;
      QueryOut o = pl.process(seqs + (size_t)q * r->S, false);
      status[q] = o.status;
      n_out[q] = (int)o.pl.size();
      for (size_t i = 0; i < o.pl.size() && (int)i < p.keep_at_most; i++) {
        OrcPlacement &d = out[(size_t)q * p.keep_at_most + i];
        d.edge = o.pl[i].edge; d.pad = 0; d.like = o.pl[i].like; d.lwr = o.pl[i].lwr;
        d.dist = o.pl[i].dist; d.pend = o.pl[i].pend;
      }
    }
  };
  if (n_threads <= 1) worker();
  else {
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; t++) th.emplace_back(worker);
    for (auto &t : th) t.join();
  }
}

// Stage-1 ranking and stage-2 trace of one query (core.ml:187-318): edges in
// rank order with scores, then the stage-2 edges tried with their like.
int orc_query_trace(void *rp, const OrcPrefs *pp, const char *seq, int *rank_edges, double *rank_scores,
                    int *n_rank, int *s2_edges, double *s2_likes, int *n_s2) {
  Ref *r = (Ref *)rp;
  Prefs p;
  p.start_pend = pp->start_pend; p.max_pend = pp->max_pend; p.initial_tolerance = pp->initial_tolerance;
  p.max_strikes = pp->max_strikes; p.strike_box = pp->strike_box; p.max_pitches = pp->max_pitches;
  p.keep_at_most = pp->keep_at_most; p.keep_factor = pp->keep_factor;
  Placer pl(*r, p);
  QueryOut o = pl.process(seq, true);
  *n_rank = (int)o.ranking.size();
  for (size_t i = 0; i < o.ranking.size(); i++) { rank_edges[i] = o.ranking[i].first; rank_scores[i] = o.ranking[i].second; }
  *n_s2 = (int)o.stage2.size();
  for (size_t i = 0; i < o.stage2.size(); i++) { s2_edges[i] = o.stage2[i].first; s2_likes[i] = o.stage2[i].second; }
  return o.status;
}

// One location optimised from (pend0, dist0) at tolerance tol: out =
// like, pend, dist.  Returns 0, or 2 (GSL error after the retry), 4 (start failure).
int orc_optimize_location(void *rp, const OrcPrefs *pp, const char *seq, int loc, double pend0, double dist0,
                          double tol, double *out) {
  Ref *r = (Ref *)rp;
  Prefs p;
  p.start_pend = pp->start_pend; p.max_pend = pp->max_pend; p.initial_tolerance = pp->initial_tolerance;
  p.max_strikes = pp->max_strikes; p.strike_box = pp->strike_box; p.max_pitches = pp->max_pitches;
  p.keep_at_most = pp->keep_at_most; p.keep_factor = pp->keep_factor;
  Placer pl(*r, p);
  pl.trial_loc = loc; pl.trial_pend = pend0; pl.trial_dist = dist0; pl.trial_tol = tol;
  QueryOut o = pl.process(seq, false);
  if (o.status) return o.status;
  out[0] = o.pl[0].like; out[1] = o.pl[0].pend; out[2] = o.pl[0].dist;
  return 0;
}

// FP64 logL and derivatives (see Placer::derivs).
int orc_loglike_derivs(void *rp, const char *seq, int loc, double pend, double dist, double *out) {
  Ref *r = (Ref *)rp;
  Prefs p;
  Placer pl(*r, p);
  return pl.derivs(seq, loc, pend, dist, out);
}

}  // extern "C"
