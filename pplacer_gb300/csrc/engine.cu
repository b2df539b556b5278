// Batched placement engine (sm_103a).
//
// Device layout (HBM):
//   darr, parr, snode : float [n_nodes][n_sites][planes][n_states]   site-major,
//                       one site of all rate planes is contiguous (64 B for DNA G4)
//   dexp, pexp, sexp  : int32 [n_nodes][n_sites] exact per-site scaling exponents
//   B3, BX            : bf16 [3][prim][n_edges][Sp], [2][n_edges][Sp] stage-1 tables
//                       (log-likelihood terms, rebased exponent digits)
//   queries           : codes, masked-site index lists (reind) and codes, lengths
//
// Pipeline of one placement call (pplacer_src/core.ml:113-409):
//   query prep -> stage-1 log table (once per start_pend) -> stage-1 scores
//   on the tensor cores -> per-query ranking -> whole-query stage 2, keep,
//   refinement and like_weight_ratio (or baseball rounds of per-trial
//   launches) -> output.
#include <math.h>

#include <cmath>

#include <algorithm>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "pgb_common.cuh"
#include "qng_rules.h"
#include "stage1_tc.cuh"
#include "tc.cuh"

namespace pgb {
namespace {

constexpr double kLn2 = 0.69314718055994530942;

enum { ST_OK = 0, ST_MAXITER = 1, ST_FAILED = 2, ST_STARTFAIL = 3 };
enum { BR_OK = 0, BR_GSLERR = 1, BR_MAXITER = 2, BR_STARTFAIL = 3 };

// ---------------------------------------------------------------------------
// Precompute kernels (FP64): like_stree.ml:43-110, pplacer_run.ml:332-340
// ---------------------------------------------------------------------------

// P_m(t) = X diag(exp(rate_m t lambda)) Xit^T for every node (diagd.ml:79-98,
// exp((rate * bl) * l_k) then dediagonalize's (l_k X_ik) Xit_jk order).
__global__ void k_node_pmats(double *pm, const double *__restrict__ bl, double scale, int n_nodes, int NM, int K,
                             const double *__restrict__ X, const double *__restrict__ Xit,
                             const double *__restrict__ lam, const double *__restrict__ rates) {
  long n = (long)n_nodes * NM * K * K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int j = (int)(t % K);
    int i = (int)((t / K) % K);
    int m = (int)((t / (K * K)) % NM);
    long node = t / ((long)K * K * NM);
    double rb = rates[m] * (bl[node] * scale);
    double acc = 0;
    for (int k = 0; k < K; k++) acc += exp(rb * lam[k]) * X[i * K + k] * Xit[j * K + k];
    pm[t] = acc;
  }
}

// Pull the per-site exponent when the site's max (over planes and states) has
// frexp exponent below thr (gmix_model.ml:163-187, gcat_model.ml:195-212).
__device__ __forceinline__ void pull_site(double *v, int n, int *e, int thr) {
  double mx = v[0];
  for (int i = 1; i < n; i++) mx = fmax(mx, v[i]);
  int te;
  frexp(mx, &te);
  if (te < thr) {
    double f = ldexp(0.5, -te + 1);
    for (int i = 0; i < n; i++) v[i] *= f;
    *e += te;
  }
}

// evolve one site of all planes: out[r][k] = sum_j P_m[k][j] in[r][j]
__device__ __forceinline__ void evolve_site(double *out, const double *in, const double *pm_node, int RP, int K,
                                            int gcat_cat) {
  for (int r = 0; r < RP; r++) {
    int m = gcat_cat >= 0 ? gcat_cat : r;
    const double *P = pm_node + (long)m * K * K;
    for (int k = 0; k < K; k++) {
      double acc = 0;
      for (int j = 0; j < K; j++) acc += P[k * K + j] * in[r * K + j];
      out[r * K + k] = acc;
    }
  }
}

struct PreCtx {
  int S, RP, K, NM, gcat;
  const uint8_t *site_cat;
  const double *lvd;     // [ncode][K]
  const double *pm;      // [n_nodes][NM][K][K] at bl
  const double *pmh;     // at bl/2
  const double *statd;
  double *distal, *evd, *prox;  // [n_nodes][S][RP][K]
  int *de, *ee, *pe;            // [n_nodes][S]
};

// Leaves: distal = LV broadcast to every plane, evd = P distal.
__global__ void k_leaves(PreCtx c, const int *__restrict__ leaves, int n_leaves, const uint8_t *__restrict__ codes) {
  long n = (long)n_leaves * c.S;
  int RK = c.RP * c.K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int li = (int)(t / c.S), s = (int)(t - (long)li * c.S);
    int node = leaves[li];
    long base = ((long)node * c.S + s) * RK;
    int code = codes[(long)li * c.S + s];
    for (int r = 0; r < c.RP; r++)
      for (int k = 0; k < c.K; k++) c.distal[base + r * c.K + k] = c.lvd[code * c.K + k];
    c.de[(long)node * c.S + s] = 0;
    c.ee[(long)node * c.S + s] = 0;
    evolve_site(c.evd + base, c.distal + base, c.pm + (long)node * c.NM * c.K * c.K, c.RP, c.K,
                c.gcat ? c.site_cat[s] : -1);
  }
}

// One post-order level: distal = product of children's evd in child order,
// pull at -50, evd = P(bl) distal (like_stree.ml:43-69).
__global__ void k_distal_level(PreCtx c, const int *__restrict__ nodes, int n_nodes_lvl,
                               const int *__restrict__ ch_start, const int *__restrict__ ch_list) {
  long n = (long)n_nodes_lvl * c.S;
  int RK = c.RP * c.K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int ni = (int)(t / c.S), s = (int)(t - (long)ni * c.S);
    int node = nodes[ni];
    long base = ((long)node * c.S + s) * RK;
    double *d = c.distal + base;
    int c0 = ch_list[ch_start[node]];
    int e = c.ee[(long)c0 * c.S + s];
    long b0 = ((long)c0 * c.S + s) * RK;
    for (int i = 0; i < RK; i++) d[i] = c.evd[b0 + i];
    for (int ci = ch_start[node] + 1; ci < ch_start[node + 1]; ci++) {
      int ch = ch_list[ci];
      long bc = ((long)ch * c.S + s) * RK;
      for (int i = 0; i < RK; i++) d[i] = d[i] * c.evd[bc + i];
      e += c.ee[(long)ch * c.S + s];
    }
    pull_site(d, RK, &e, -50);
    c.de[(long)node * c.S + s] = e;
    c.ee[(long)node * c.S + s] = e;
    evolve_site(c.evd + base, d, c.pm + (long)node * c.NM * c.K * c.K, c.RP, c.K, c.gcat ? c.site_cat[s] : -1);
  }
}

// One pre-order level: prox[child] = P(bl_parent) prox[parent] times the
// siblings' evd in child order, pull at -50 (like_stree.ml:74-100).
__global__ void k_prox_level(PreCtx c, const int *__restrict__ nodes, int n_nodes_lvl, const int *__restrict__ parent,
                             const int *__restrict__ ch_start, const int *__restrict__ ch_list) {
  long n = (long)n_nodes_lvl * c.S;
  int RK = c.RP * c.K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int ni = (int)(t / c.S), s = (int)(t - (long)ni * c.S);
    int node = nodes[ni];
    int p = parent[node];
    long base = ((long)node * c.S + s) * RK;
    double *out = c.prox + base;
    evolve_site(out, c.prox + ((long)p * c.S + s) * RK, c.pm + (long)p * c.NM * c.K * c.K, c.RP, c.K,
                c.gcat ? c.site_cat[s] : -1);
    int e = c.pe[(long)p * c.S + s];
    for (int ci = ch_start[p]; ci < ch_start[p + 1]; ci++) {
      int sib = ch_list[ci];
      if (sib == node) continue;
      long bs = ((long)sib * c.S + s) * RK;
      for (int i = 0; i < RK; i++) out[i] = out[i] * c.evd[bs + i];
      e += c.ee[(long)sib * c.S + s];
    }
    pull_site(out, RK, &e, -50);
    c.pe[(long)node * c.S + s] = e;
  }
}

__global__ void k_set_unit(double *g, int *e, long n_vals, long n_exps) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n_vals; t += (long)gridDim.x * blockDim.x) {
    g[t] = 1.0;
    if (t < n_exps) e[t] = 0;
  }
}

// Pull at -10, supernode = statd (P(bl/2) d) (P(bl/2) p), FP32 copies
// (pplacer_run.ml:332-340, glv_arr.ml:46-57).
__global__ void k_finish_glvs(PreCtx c, int n_nodes, float *d32, float *p32, float *s32, int *dexp, int *pexp,
                              int *sexp) {
  long n = (long)n_nodes * c.S;
  int RK = c.RP * c.K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int node = (int)(t / c.S), s = (int)(t - (long)node * c.S);
    long base = t * RK;
    double *d = c.distal + base, *p = c.prox + base;
    int ed = c.de[t], ep = c.pe[t];
    pull_site(d, RK, &ed, -10);
    pull_site(p, RK, &ep, -10);
    dexp[t] = ed;
    pexp[t] = ep;
    int cat = c.gcat ? c.site_cat[s] : -1;
    const double *P = c.pmh + (long)node * c.NM * c.K * c.K;
    for (int r = 0; r < c.RP; r++) {
      int m = cat >= 0 ? cat : r;
      const double *Pm = P + (long)m * c.K * c.K;
      for (int k = 0; k < c.K; k++) {
        double ud = 0, up = 0;
        for (int j = 0; j < c.K; j++) {
          ud += Pm[k * c.K + j] * d[r * c.K + j];
          up += Pm[k * c.K + j] * p[r * c.K + j];
        }
        s32[base + r * c.K + k] = (float)(c.statd[k] * ud * up);
        d32[base + r * c.K + k] = (float)d[r * c.K + k];
        p32[base + r * c.K + k] = (float)p[r * c.K + k];
      }
    }
    sexp[t] = ed + ep;
  }
}

// Site-category refinement (gcat_model.ml:387-419), one category pass: the
// per-site tree log likelihood from the root's distal GLV (the product of
// its children's evolved GLVs, Like_stree.site_log_like_arr), scored
// ll + 2 log(rate) - 3 rate; a site keeps the first category with the
// highest score.
__global__ void k_refine_site(const double *__restrict__ root_distal, const int *__restrict__ root_e,
                              const double *__restrict__ statd, int S, int K, int cat, double bonus, double *best,
                              int *best_cat) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
    double u = 0;
    for (int k = 0; k < K; k++) u += statd[k] * root_distal[(long)s * K + k];
    double x = log(u) + kLn2 * root_e[s] + bonus;
    if (x > best[s]) { best[s] = x; best_cat[s] = cat; }
  }
}

__global__ void k_refine_init(double *best, int *best_cat, int S) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
    best[s] = -INFINITY;
    best_cat[s] = -1;
  }
}

// Caller-provided FP64 GLVs [node][R][S][K] -> FP32 site-major.
__global__ void k_import_glv(const double *__restrict__ src, const int *__restrict__ se, float *dst, int *de,
                             int n_nodes, int S, int RP, int K) {
  long n = (long)n_nodes * RP * S * K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int k = (int)(t % K);
    int s = (int)((t / K) % S);
    int r = (int)((t / ((long)K * S)) % RP);
    long node = t / ((long)K * S * RP);
    dst[((node * S + s) * RP + r) * K + k] = (float)src[t];
    if (r == 0 && k == 0) de[node * S + s] = se[node * S + s];
  }
}

// Supernodes from FP64 darr/parr in the caller's [node][R][S][K] layout.
__global__ void k_snodes_from(const double *__restrict__ d, const double *__restrict__ p, const int *__restrict__ de,
                              const int *__restrict__ pe, const double *__restrict__ pmh,
                              const double *__restrict__ statd, const uint8_t *__restrict__ site_cat, int gcat,
                              float *s32, int *sexp, int n_nodes, int S, int RP, int K, int NM) {
  long n = (long)n_nodes * S;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    long node = t / S;
    int s = (int)(t - node * S);
    for (int r = 0; r < RP; r++) {
      int m = gcat ? site_cat[s] : r;
      const double *Pm = pmh + (node * NM + m) * K * K;
      const double *dv = d + ((node * RP + r) * S + s) * K, *pv = p + ((node * RP + r) * S + s) * K;
      for (int k = 0; k < K; k++) {
        double ud = 0, up = 0;
        for (int j = 0; j < K; j++) {
          ud += Pm[k * K + j] * dv[j];
          up += Pm[k * K + j] * pv[j];
        }
        s32[(t * RP + r) * K + k] = (float)(statd[k] * ud * up);
      }
    }
    sexp[t] = de[t] + pe[t];
  }
}

// ---------------------------------------------------------------------------
// Query preparation: character codes, informative mask, masked site lists
// (core.ml:121-170).  One CTA per query.
// ---------------------------------------------------------------------------
// Columns are visited in the order `order` (null: 0 .. S-1); the CAT models
// pass the columns grouped by category, so that a query's informative sites
// come grouped by category and neighbouring trial threads read the same
// category's matrices (the site order changes only FP32 summation order).
// The packed word of a site is (category << 24) | (column << 8) | code, the
// category byte from site_cat (CAT models) or 0.
__global__ void k_query_prep(const char *__restrict__ seqs, int S, int prim, const uint8_t *__restrict__ char_code,
                             const uint8_t *__restrict__ informative, const uint16_t *__restrict__ order,
                             const uint8_t *__restrict__ site_cat, uint8_t *qcode, uint16_t *reind, uint8_t *mcode,
                             uint32_t *rcode, int *qlen, int *qstatus, int *qamb) {
  int q = blockIdx.x;
  const char *seq = seqs + (long)q * S;
  __shared__ int s_off;
  __shared__ int s_bad;
  __shared__ int s_amb;
  __shared__ int s_warp[32];
  if (threadIdx.x == 0) { s_off = 0; s_bad = 0; s_amb = 0; }
  __syncthreads();
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < S; base += blockDim.x) {
    int s = base + threadIdx.x;
    if (order && s < S) s = order[s];
    uint8_t c = kBadCode;
    int inf = 0;
    if (s < S) {
      c = char_code[(uint8_t)seq[s]];
      if (c == kBadCode) atomicOr(&s_bad, 1);
      else inf = informative[c];
      if (inf && c >= prim) atomicAdd(&s_amb, 1);
      qcode[(long)q * S + s] = c;
    }
    unsigned bal = __ballot_sync(0xffffffffu, inf);
    if (lane == 0) s_warp[w] = __popc(bal);
    __syncthreads();
    int before = 0, tot = 0;
    for (int i = 0; i < nw; i++) {
      if (i < w) before += s_warp[i];
      tot += s_warp[i];
    }
    if (inf) {
      int pos = s_off + before + __popc(bal & ((1u << lane) - 1u));
      reind[(long)q * S + pos] = (uint16_t)s;
      mcode[(long)q * S + pos] = c;
      rcode[(long)q * S + pos] = (site_cat ? (uint32_t)site_cat[s] << 24 : 0u) | ((uint32_t)s << 8) | c;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_off += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    qlen[q] = s_off;
    qamb[q] = s_amb;
    qstatus[q] = s_bad ? PGB_Q_BAD_CHAR : (s_off == 0 ? PGB_Q_NO_INFORMATIVE : PGB_Q_OK);
  }
}

// ---------------------------------------------------------------------------
// Stage 1 (core.ml:187-197, Glv.masked_logdot against every supernode): the
// edge-side tables here, the contraction on the tensor cores in
// stage1_tc.cuh (k_s1_mma), FP64 scores and ambiguity characters in
// k_s1_scores.
// ---------------------------------------------------------------------------
struct S1Ctx {
  int S, Sp, RP, K, NM, gcat, ncode, prim, n_edges;
  const float *snode;        // [n_nodes][S][RP][K]
  const int *sexp;           // [n_nodes][S]
  const int *edge_nodes;     // [n_edges]
  const float *qe;           // [NM][ncode][K] evolved query LV per character
  const uint8_t *site_cat;
};

__device__ __forceinline__ float s1_util(const S1Ctx &c, int node, int s, int code) {
  const float *sn = c.snode + ((long)node * c.S + s) * c.RP * c.K;
  float u = 0.f;
  for (int r = 0; r < c.RP; r++) {
    int m = c.gcat ? c.site_cat[s] : r;
    const float *q = c.qe + ((long)m * c.ncode + code) * c.K;
    for (int k = 0; k < c.K; k++) u = fmaf(q[k], sn[r * c.K + k], u);
  }
  return u;
}

// Edge-side tables, once per start_pend, one block per edge:
//   B3[plane][code][edge][s]: T split into bf16 hi / mid / lo (plane 0..2);
//   BX[digit][edge][s]: the exponents rebased by the edge's mean,
//     ex - base = 256 hi + lo with lo in [0, 255], as 256 hi and lo (exact in
//     bf16 while |ex - base| < 2^15);
//   ebase[edge] = base.
// err is set when an edge breaks the exactness bounds of the exponent sums
// (a per-site deviation of 2^15 or more, or digit sums reaching 2^24).
__global__ void __launch_bounds__(256) k_s1_tables(S1Ctx c, __nv_bfloat16 *B3, __nv_bfloat16 *BX, int *ebase,
                                                   int *err) {
  __shared__ long long sh[8];
  const int ei = blockIdx.x;
  const int node = c.edge_nodes[ei];
  const int *ex = c.sexp + (long)node * c.S;
  long long sum = 0;
  for (int s = threadIdx.x; s < c.S; s += blockDim.x) sum += ex[s];
  sum = s1::block_sum_ll(sum, sh);
  long long b = sum / c.S;
  if (b * c.S > sum) b--;  // floor of the mean
  const int base = (int)b;
  const size_t plane = (size_t)c.prim * c.n_edges * c.Sp;
  long long digits = 0;
  int bad = 0;
  for (int s = threadIdx.x; s < c.S; s += blockDim.x) {
    for (int code = 0; code < c.prim; code++) {
      double lg = log((double)s1_util(c, node, s, code));
      if (!(lg > -1e30)) lg = -1e30;  // log 0 (and NaN) -> a finite -1e30: 0 * inf would poison the sums
      if (lg > 1e30) lg = 1e30;
      const float v = (float)lg;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(hi);
      const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
      const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
      const size_t o = ((size_t)code * c.n_edges + ei) * c.Sp + s;
      B3[o] = hi;
      B3[plane + o] = mid;
      B3[2 * plane + o] = lo;
    }
    const int d = ex[s] - base;
    bad |= d >= 32768 || d < -32768;
    const int dh = d >> 8;          // floor(d / 256)
    const int dl = d - (dh << 8);   // 0..255
    digits += 256LL * (dh < 0 ? -dh : dh) + dl;
    BX[(size_t)ei * c.Sp + s] = __float2bfloat16_rn(256.f * (float)dh);
    BX[(size_t)c.n_edges * c.Sp + (size_t)ei * c.Sp + s] = __float2bfloat16_rn((float)dl);
  }
  digits = s1::block_sum_ll(digits, sh);
  const long long nbad = s1::block_sum_ll(bad, sh);
  if (threadIdx.x == 0) {
    ebase[ei] = base;
    // the epilogue's int32 total, base * n_q + digit sum, stays exact
    if (nbad || digits >= s1::kMaxExpDigitSum || (b < 0 ? -b : b) * c.S >= (1LL << 30)) atomicExch(err, 1);
  }
}

// FP64 scores of the n_rows listed queries: the tensor-core pair plus, when
// `ambig`, the logs of the site likelihoods of their ambiguity characters.
__global__ void k_s1_scores(S1Ctx c, int n_rows, const int *__restrict__ qlist, int ambig,
                            const uint16_t *__restrict__ reind, const uint8_t *__restrict__ mcode,
                            const int *__restrict__ qlen, const int *__restrict__ qstatus,
                            const int2 *__restrict__ pairs, double log_nrates, double *scores) {
  const int row = blockIdx.x;
  if (row >= n_rows) return;
  const int q = qlist[row];
  const int ei = blockIdx.y * blockDim.x + threadIdx.x;
  if (ei >= c.n_edges || qstatus[q] != PGB_Q_OK) return;
  const int node = c.edge_nodes[ei];
  double acc = 0;
  if (ambig)
    for (int i = 0; i < qlen[q]; i++) {
      const int code = mcode[(long)q * c.S + i];
      if (code >= c.prim) acc += log((double)s1_util(c, node, reind[(long)q * c.S + i], code));
    }
  const long o = (long)q * c.n_edges + ei;
  scores[o] = s1::s1_pair_score(pairs[o], s1::s1_qconst(qlen[q], log_nrates)) + acc;
}

// Per-query ranking: edges by score, descending, ties to the lower edge index
// (stable sort of the ascending edge list, fig.ml:143-147); NaN sorts below
// every number as OCaml's compare does.  Scores map to order-preserving
// 64-bit keys.  Only the rk best edges are needed, so each query takes one
// warp and extracts them by repeated arg-max: lane L owns edges L, L + 32,
// ... and keeps its best remaining (key, edge); the warp's winner is the
// arg-max over lanes (an xor butterfly, identical in every lane), and only
// the winner's owner lane marks it taken and rescans its edges.
__device__ __forceinline__ unsigned long long s1_key(double v) {
  if (isnan(v)) return 0ull;
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Each lane keeps a sorted cache of its kRankCache best remaining edges; a
// lane that wins pops its cache and, when it runs dry, refills it from its
// edges ranked after the last one it gave out.  With rk well below
// 32 * kRankCache most lanes scan their edges once, reading the scores
// straight from global memory; ranking many edges per query
// (rk = E when every edge is tried) stages the row's keys in shared memory
// first, as the refills rescan it.
constexpr int kRankCache = 8;

__device__ __forceinline__ bool rank_before(unsigned long long ka, int ia, unsigned long long kb, int ib) {
  return ka > kb || (ka == kb && ia < ib);
}

// The FP64 score of (q, i): formed from the tensor-core pair, or read from
// the FP64 row of a query with ambiguity characters.
struct S1Scores {
  const int2 *pairs;
  const double *scores;
  const int *qlen, *qamb;
  double log_nrates;
};

// Top-rk extraction of one warp over the edges i with use(i): each lane
// keeps a sorted cache of its kRankCache best remaining edges and refills it
// from its edges ranked after the last one it gave out; the warp's winner of
// each round is the arg-max over the lanes' heads (an xor butterfly, the
// same in every lane).  out(r, i, key) is called in every lane for each
// round r (i < 0 when fewer than rk edges are used).
template <typename KeyFn, typename UseFn, typename OutFn>
__device__ __forceinline__ void warp_topk(int E, int rk, int lane, KeyFn key_of, UseFn use, OutFn out) {
  unsigned long long ck[kRankCache];
  int ci[kRankCache];
  unsigned long long lk = 0ull;  // last edge this lane gave out (li < 0: none yet)
  int li = -1;
  auto refill = [&]() {  // the kRankCache best of the lane's edges ranked after (lk, li)
#pragma unroll
    for (int c = 0; c < kRankCache; c++) { ck[c] = 0ull; ci[c] = -1; }
    for (int i = lane; i < E; i += 32) {
      if (!use(i)) continue;
      unsigned long long k = key_of(i);
      if (li >= 0 && !rank_before(lk, li, k, i)) continue;
      if (ci[kRankCache - 1] >= 0 && !rank_before(k, i, ck[kRankCache - 1], ci[kRankCache - 1])) continue;
      // insert into the sorted cache
      unsigned long long kk = k;
      int ii = i;
#pragma unroll
      for (int c = 0; c < kRankCache; c++) {
        if (ci[c] < 0 || rank_before(kk, ii, ck[c], ci[c])) {
          unsigned long long tk = ck[c];
          int ti = ci[c];
          ck[c] = kk; ci[c] = ii;
          kk = tk; ii = ti;
        }
      }
    }
  };
  refill();
  for (int r = 0; r < rk; r++) {
    unsigned long long wk = ck[0];
    int wi = ci[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ok = __shfl_xor_sync(0xffffffffu, wk, o);
      int oi = __shfl_xor_sync(0xffffffffu, wi, o);
      if (oi >= 0 && (wi < 0 || rank_before(ok, oi, wk, wi))) { wk = ok; wi = oi; }
    }
    out(r, wi, wk);
    if (wi >= 0 && wi == ci[0]) {  // this lane's head: pop it
      lk = ck[0];
      li = ci[0];
#pragma unroll
      for (int c = 0; c + 1 < kRankCache; c++) { ck[c] = ck[c + 1]; ci[c] = ci[c + 1]; }
      ck[kRankCache - 1] = 0ull;
      ci[kRankCache - 1] = -1;
      if (ci[0] < 0) refill();
    }
  }
}

// Ranking of one query per warp by the stage-1 score of each edge (a query
// with ambiguity characters reads its FP64 row; the others form the score
// from the tensor-core pair as s1::s1_pair_df, in FP32 arithmetic, which
// FP64's slow rate on this part makes the cheaper key).
__global__ void __launch_bounds__(128) k_rank_warp(S1Scores sv, int E, int rk, int Q,
                                                   const int *__restrict__ qstatus, int *rank, int keys_in_smem) {
  extern __shared__ unsigned long long rk_smem[];
  const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = blockIdx.x * nw + w;
  if (q >= Q || qstatus[q] != PGB_Q_OK) return;
  unsigned long long *keys = rk_smem + (long)w * E;
  const bool amb = sv.qamb[q] > 0;
  const double *sc = sv.scores + (long)q * E;
  const int2 *pr = sv.pairs + (long)q * E;
  const s1::QConst qc = s1::s1_qconst(sv.qlen[q], sv.log_nrates);
  auto key_of = [&](int i) { return amb ? s1_key(sc[i]) : s1::s1_pair_key(pr[i], qc); };
  int *out_row = rank + (long)q * rk;
  auto write = [&](int r, int i, unsigned long long) {
    if (lane == 0) out_row[r] = i;
  };
  auto all = [](int) { return true; };
  if (keys_in_smem) {
    for (int i = lane; i < E; i += 32) keys[i] = key_of(i);
    __syncwarp();
    warp_topk(E, rk, lane, [&](int i) { return keys[i]; }, all, write);
    return;
  }
  warp_topk(E, rk, lane, key_of, all, write);
}

#include "trials.cuh"
#include "trials_warp.cuh"
#include "trials_tc.cuh"

// ---------------------------------------------------------------------------
// Baseball (core.ml:283-318) and keep / refine / like_weight_ratio
// (core.ml:336-377, ppatteries.ml:175-183, pquery.ml:8-9,92).
// ---------------------------------------------------------------------------
struct BBState {
  int next, strikes, nres, done;
  double record;
};
struct ResEntry {
  int edge, status;
  double like, pend, dist;
  EvalOut ev;  // the trial's evaluation at (pend, dist): seeds the Newton refinement
};
struct BBCtx {
  int Q, rk, maxr, n_edges, bins;
  const int *rank;            // [Q][rk] edge indices
  const int *edge_nodes;
  const double *bl;
  const int *qlen;
  int *qstatus;
  BBState *bb;
  ResEntry *res;              // [Q][maxr]
  int *tbase, *tcount;        // [Q]
  TrialIn *trials;
  int *bin_count;             // [bins]
  int *bin_list;              // [bins][cap_trials]
  const int *bin_limit;       // [bins] max Sq of each bin
  int cap_trials;
  int *n_active;
  double start_pend, tol, strike_box;
  long max_pitches, max_strikes;
};

__device__ int bin_of(const BBCtx &c, int sq) {
  for (int b = 0; b < c.bins; b++)
    if (sq <= c.bin_limit[b]) return b;
  return c.bins - 1;
}

__global__ void k_bb_init(BBCtx c) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  BBState s;
  s.next = 0; s.strikes = 0; s.nres = 0;
  s.done = c.qstatus[q] != PGB_Q_OK;
  s.record = -INFINITY;
  c.bb[q] = s;
}

__global__ void k_bb_emit(BBCtx c, int B, int *counter) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  BBState s = c.bb[q];
  c.tcount[q] = 0;
  if (s.done) return;
  int n = min(B, c.rk - s.next);
  if (n <= 0) { c.bb[q].done = 1; return; }
  int base = atomicAdd(counter, n);
  if (base + n > c.cap_trials) { c.bb[q].done = 1; c.qstatus[q] = PGB_Q_EMPTY; return; }
  c.tbase[q] = base;
  c.tcount[q] = n;
  int bin = bin_of(c, c.qlen[q]);
  int bpos = atomicAdd(&c.bin_count[bin], n);
  for (int j = 0; j < n; j++) {
    int ei = c.rank[(long)q * c.rk + s.next + j];
    int node = c.edge_nodes[ei];
    TrialIn t{};
    t.q = q;
    t.node = node;
    t.pend0 = c.start_pend;
    t.dist0 = c.bl[node] / 2.;
    t.tol = c.tol;
    c.trials[base + j] = t;
    c.bin_list[(long)bin * c.cap_trials + bpos + j] = base + j;
  }
}

__global__ void k_bb_update(BBCtx c, const TrialRes *__restrict__ tres) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  BBState s = c.bb[q];
  int n = c.tcount[q];
  if (s.done || n == 0) return;
  int base = c.tbase[q];
  for (int j = 0; j < n && !s.done; j++) {
    TrialRes r = tres[base + j];
    int ei = c.rank[(long)q * c.rk + s.next];
    s.next++;
    if (r.status == ST_STARTFAIL) { s.done = 1; c.qstatus[q] = PGB_Q_START_FAILURE; break; }
    if (r.status == ST_FAILED) continue;  // skipped location (core.ml:286-297)
    long before = s.nres;
    if (s.nres < c.maxr) {
      ResEntry e;
      e.edge = ei; e.status = r.status; e.like = r.like; e.pend = r.pend; e.dist = r.dist; e.ev = r.last;
      c.res[(long)q * c.maxr + s.nres] = e;
      s.nres++;
    }
    if (before >= c.max_pitches) { s.done = 1; break; }
    if (r.like > s.record) s.record = r.like;
    else if (r.like < s.record - c.strike_box) {
      if (s.strikes + 1 >= c.max_strikes) { s.done = 1; break; }
      s.strikes++;
    }
  }
  if (!s.done && s.next >= c.rk) s.done = 1;
  if (!s.done) atomicAdd(c.n_active, 1);
  c.bb[q] = s;
}

// sort results by like (stable, descending), keep, emit refinement trials
__global__ void k_keep_emit(BBCtx c, int keep_at_most, double log_keep_factor, int *keep_idx, int *keep_n,
                            int *counter) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  keep_n[q] = 0;
  c.tcount[q] = 0;
  if (c.qstatus[q] != PGB_Q_OK) return;
  int n = c.bb[q].nres;
  if (n == 0) { c.qstatus[q] = PGB_Q_EMPTY; return; }
  ResEntry *r = c.res + (long)q * c.maxr;
  // insertion sort: stable, descending by like (NaN last)
  for (int i = 1; i < n; i++) {
    ResEntry x = r[i];
    int j = i - 1;
    while (j >= 0 && (isnan(r[j].like) ? !isnan(x.like) : (!isnan(x.like) && x.like > r[j].like))) {
      r[j + 1] = r[j];
      j--;
    }
    r[j + 1] = x;
  }
  double best = r[0].like;
  int nk = 0;
  for (int i = 0; i < n; i++)
    if (i < keep_at_most && r[i].like >= log_keep_factor + best) keep_idx[(long)q * keep_at_most + nk++] = i;
  keep_n[q] = nk;
  int base = atomicAdd(counter, nk);
  c.tbase[q] = base;
  c.tcount[q] = nk;
  int bin = bin_of(c, c.qlen[q]);
  int bpos = atomicAdd(&c.bin_count[bin], nk);
  for (int j = 0; j < nk; j++) {
    ResEntry e = r[keep_idx[(long)q * keep_at_most + j]];
    TrialIn t{};
    t.q = q;
    t.node = c.edge_nodes[e.edge];
    t.pend0 = e.pend;
    t.dist0 = e.dist;
    t.tol = 1e-5;  // final_tolerance (core.ml:14)
    t.seeded = 1;  // used by the Newton form only
    t.seed = e.ev;
    c.trials[base + j] = t;
    c.bin_list[(long)bin * c.cap_trials + bpos + j] = base + j;
  }
}

// Posterior probabilities (core.ml:378-401): one marginal-likelihood trial
// per kept location (Three_tax.calc_marg_prob, three_tax.ml:169-215), around
// the refined optimum (the stage-2 one where the refinement failed), at trial
// index off + tbase[q] + j.
__global__ void k_pp_emit(BBCtx c, int keep_at_most, const int *__restrict__ keep_idx,
                          const int *__restrict__ keep_n, const TrialRes *__restrict__ tres, int off, int prior_kind,
                          const double *__restrict__ prior_mu) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  const int nk = keep_n[q];
  if (c.qstatus[q] != PGB_Q_OK || nk == 0) return;
  const ResEntry *r = c.res + (long)q * c.maxr;
  const int bin = bin_of(c, c.qlen[q]);
  const int bpos = atomicAdd(&c.bin_count[bin], nk);
  for (int j = 0; j < nk; j++) {
    const ResEntry e = r[keep_idx[(long)q * keep_at_most + j]];
    const TrialRes tr = tres[c.tbase[q] + j];
    const bool ok = !(tr.status == ST_FAILED || tr.status == ST_STARTFAIL);
    TrialIn t{};
    t.q = q;
    t.node = c.edge_nodes[e.edge];
    t.pend0 = ok ? tr.pend : e.pend;
    t.dist0 = ok ? tr.dist : e.dist;
    t.tol = 1e-5;
    t.seeded = 1;
    t.seed = ok ? tr.last : e.ev;
    t.marginal = 1;
    t.prior_kind = prior_kind;
    t.prior_mu = prior_mu[t.node];
    const int ti = off + c.tbase[q] + j;
    c.trials[ti] = t;
    c.bin_list[(long)bin * c.cap_trials + bpos + j] = ti;
  }
}

// pp_off >= 0: the marginal likelihoods are the results at pp_off + tbase[q]
// + j, and give the posterior probabilities (ll_normalized_prob, core.ml:
// 396-401).
__global__ void k_finalize(BBCtx c, int keep_at_most, const int *__restrict__ keep_idx, const int *__restrict__ keep_n,
                           const TrialRes *__restrict__ tres, int pp_off, pgb_placement *out, int *n_out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.Q) return;
  int nk = keep_n[q];
  n_out[q] = 0;
  if (c.qstatus[q] != PGB_Q_OK || nk == 0) return;
  const ResEntry *r = c.res + (long)q * c.maxr;
  pgb_placement *o = out + (long)q * keep_at_most;
  double like[64];
  int m = min(nk, 64);
  for (int j = 0; j < m; j++) {
    ResEntry e = r[keep_idx[(long)q * keep_at_most + j]];
    TrialRes t = tres[c.tbase[q] + j];
    pgb_placement p;
    p.edge = c.edge_nodes[e.edge];
    p.pad = 0;
    p.marginal_like = NAN;
    p.post_prob = NAN;
    if (t.status == ST_FAILED || t.status == ST_STARTFAIL) { p.like = e.like; p.pend = e.pend; p.dist = e.dist; }
    else { p.like = t.like; p.pend = t.pend; p.dist = t.dist; }
    if (pp_off >= 0) p.marginal_like = tres[pp_off + c.tbase[q] + j].like;
    like[j] = p.like;
    o[j] = p;
  }
  for (int j = 0; j < m; j++) {
    double tot = 0;
    for (int k = 0; k < m; k++) tot += exp(like[k] - like[j]);
    o[j].lwr = 1. / tot;
  }
  if (pp_off >= 0)
    for (int j = 0; j < m; j++) {
      double tot = 0;
      for (int k = 0; k < m; k++) tot += exp(o[k].marginal_like - o[j].marginal_like);
      o[j].post_prob = 1. / tot;
    }
  for (int i = 1; i < m; i++) {  // stable sort by lwr, descending
    pgb_placement x = o[i];
    int j = i - 1;
    while (j >= 0 && x.lwr > o[j].lwr) { o[j + 1] = o[j]; j--; }
    o[j + 1] = x;
  }
  n_out[q] = m;
}

// ---------------------------------------------------------------------------
// Whole queries, one per team -- a warp (nucleotide Gamma mixtures), a
// tensor-core CTA (20 states) or a CUDA-core CTA: the baseball search over
// the stage-1 ranking (core.ml:283-318), keep (core.ml:336-352), refinement
// from the kept optima (core.ml:353-377), the marginal likelihoods with
// calc_pp and like_weight_ratio (pquery.ml:8-9).  A query's trials run in
// rank order inside its team, each decided before the next starts, so
// nothing is evaluated speculatively and no host round trip separates the
// trials; queries come from a counter, longest first.  The decisions are
// those of k_bb_update / k_keep_emit / k_finalize for one result at a time.
// ---------------------------------------------------------------------------
struct PlaceCtx {
  BBCtx bb;
  int calc_pp, prior_kind;  // prior_kind: 0 uniform, 1 exponential with per-node mean prior_mu
  const double *prior_mu;
  const int *qorder;  // queries, longest first
  int *qnext;         // next position in qorder
  int keep_at_most;
  double log_keep_factor;
  pgb_placement *out;  // [Q][keep_at_most]
  int *n_out;
  unsigned long long *tstats;  // [0] baseball trials, [1] refinement trials
};

// The whole-query search for any team of threads that runs
// one trial at a time: Team::leader() is the one thread that writes results,
// Team::sync() orders its writes before the team's reads, Team::bcast(v) is
// the leader's v in every thread, Team::trial(t) the trial's result
// (identical in every thread) and Team::aborted() true after a trial the
// team could not complete (the launch then reports an error).
template <class Team>
__device__ __forceinline__ void place_queries(Team &tm, const TrialCtx &c, const PlaceCtx &p) {
  const BBCtx &b = p.bb;
  // One trial call site (the trial code is inlined once): a query moves from
  // its baseball trials (refine < 0) to the refinement of its kept
  // locations (refine = index of the next one).
  int q = -1, next = 0, nres = 0, nk = 0, refine = -1;
  bool marginal = false;  // the next trial is the marginal likelihood of kept location `refine`
  long strikes = 0;
  double record = -INFINITY, pend_hint = b.start_pend;
  unsigned long long n_bb = 0;
  for (;;) {
    if (q < 0) {  // take the next query
      const int qi = tm.bcast(tm.leader() ? atomicAdd(p.qnext, 1) : 0);
      if (qi >= b.Q) break;
      q = p.qorder[qi];
      if (tm.leader()) p.n_out[q] = 0;
      if (b.qstatus[q] != PGB_Q_OK || b.rk < 1) { q = -1; continue; }
      next = 0; nres = 0; nk = 0; refine = -1; strikes = 0; record = -INFINITY; n_bb = 0; marginal = false;
      pend_hint = b.start_pend;
    }
    ResEntry *r = b.res + (long)q * b.maxr;
    TrialIn t{};
    t.q = q;
    int ei = -1;
    if (refine < 0) {
      ei = b.rank[(long)q * b.rk + next];
      t.node = b.edge_nodes[ei];
      // The Newton form starts the pendant length at the query's best
      // optimum so far (the optimum, not the path, is its result); the
      // Brent replica keeps the reference's start.
      t.pend0 = c.optimizer == 1 ? pend_hint : b.start_pend;
      t.dist0 = b.bl[t.node] / 2.;
      t.tol = b.tol;
    } else {
      const ResEntry e = r[refine];
      t.node = b.edge_nodes[e.edge];
      t.pend0 = e.pend;
      t.dist0 = e.dist;
      t.tol = 1e-5;  // final_tolerance (core.ml:14)
      t.seeded = 1;  // the evaluation at (pend0, dist0); the Newton form does not redo it
      t.seed = e.ev;
      if (marginal) {  // after the refinement: e holds the refined optimum
        t.marginal = 1;
        t.prior_kind = p.prior_kind;
        t.prior_mu = p.prior_mu[t.node];
      }
    }
    const TrialRes tr = tm.trial(t);
    if (tm.aborted()) return;
    if (refine >= 0) {  // ---- a refined location, or its marginal likelihood ----
      pgb_placement *o = p.out + (long)q * p.keep_at_most;
      if (marginal) {
        if (tm.leader()) o[refine].marginal_like = tr.like;
        marginal = false;
      } else {
        const bool ok = !(tr.status == ST_FAILED || tr.status == ST_STARTFAIL);
        if (tm.leader()) {
          ResEntry e = r[refine];
          pgb_placement pl;
          pl.edge = t.node;
          pl.pad = 0;
          pl.lwr = 0;
          pl.marginal_like = NAN;
          pl.post_prob = NAN;
          if (!ok) { pl.like = e.like; pl.pend = e.pend; pl.dist = e.dist; }
          else { pl.like = tr.like; pl.pend = tr.pend; pl.dist = tr.dist; }
          o[refine] = pl;
          if (ok && p.calc_pp) {  // the marginal likelihood integrates around the refined optimum
            e.pend = tr.pend; e.dist = tr.dist; e.ev = tr.last;
            r[refine] = e;
          }
        }
        tm.sync();
        if (p.calc_pp) {
          marginal = true;
          continue;
        }
      }
      if (++refine < nk) continue;
      // like_weight_ratio (and with calc_pp the posterior probabilities,
      // core.ml:396-401), then stable sort by like_weight_ratio, descending
      if (tm.leader()) {
        atomicAdd(&p.tstats[1], (unsigned long long)nk);
        const int m = min(nk, 64);
        for (int j = 0; j < m; j++) {
          double tot = 0;
          for (int k = 0; k < m; k++) tot += exp(o[k].like - o[j].like);
          o[j].lwr = 1. / tot;
        }
        if (p.calc_pp)
          for (int j = 0; j < m; j++) {
            double tot = 0;
            for (int k = 0; k < m; k++) tot += exp(o[k].marginal_like - o[j].marginal_like);
            o[j].post_prob = 1. / tot;
          }
        for (int i = 1; i < m; i++) {
          pgb_placement x = o[i];
          int j = i - 1;
          while (j >= 0 && x.lwr > o[j].lwr) { o[j + 1] = o[j]; j--; }
          o[j + 1] = x;
        }
        p.n_out[q] = m;
      }
      tm.sync();
      q = -1;
      continue;
    }
    // ---- a baseball result (k_bb_update's rules for one trial) ----
    n_bb++;
    next++;
    bool stop = false;
    int qst = PGB_Q_OK;
    if (tr.status == ST_STARTFAIL) {
      qst = PGB_Q_START_FAILURE;
      stop = true;
    } else if (tr.status != ST_FAILED) {  // ST_FAILED: skipped location (core.ml:286-297)
      const long before = nres;
      if (nres < b.maxr) {
        if (tm.leader()) {
          ResEntry e;
          e.edge = ei; e.status = tr.status; e.like = tr.like; e.pend = tr.pend; e.dist = tr.dist; e.ev = tr.last;
          r[nres] = e;
        }
        nres++;
      }
      if (before >= b.max_pitches) stop = true;
      else if (tr.like > record) {
        record = tr.like;
        if (tr.pend > 1e-6 && tr.pend < c.max_pend) pend_hint = tr.pend;
      }
      else if (tr.like < record - b.strike_box) {
        if (strikes + 1 >= b.max_strikes) stop = true;
        else strikes++;
      }
    }
    if (!stop && next < b.rk) continue;
    if (tm.leader()) atomicAdd(&p.tstats[0], n_bb);
    if (qst != PGB_Q_OK || nres == 0) {
      if (tm.leader()) b.qstatus[q] = qst != PGB_Q_OK ? qst : PGB_Q_EMPTY;
      tm.sync();
      q = -1;
      continue;
    }
    // ---- keep: stable sort by like, descending, NaN last ----
    tm.sync();
    if (tm.leader())
      for (int i = 1; i < nres; i++) {
        ResEntry x = r[i];
        int j = i - 1;
        while (j >= 0 && (isnan(r[j].like) ? !isnan(x.like) : (!isnan(x.like) && x.like > r[j].like))) {
          r[j + 1] = r[j];
          j--;
        }
        r[j + 1] = x;
      }
    tm.sync();
    const double best = r[0].like;
    nk = 0;
    while (nk < nres && nk < p.keep_at_most && r[nk].like >= p.log_keep_factor + best) nk++;
    if (nk == 0) { q = -1; continue; }
    refine = 0;
  }
}

// A warp as a team (nucleotide Gamma mixtures, CAT): lane 0 leads.
template <int RP, bool CAT, int EIG = 0>
struct WarpTeam {
  static constexpr bool kEig = EIG != 0;
  const TrialCtx &c;
  const TrialSmem &sm;
  float4 *ring;
  int lane;
  __device__ bool leader() const { return lane == 0; }
  __device__ void sync() const { __syncwarp(); }
  __device__ int bcast(int v) const { return __shfl_sync(0xffffffffu, v, 0); }
  __device__ TrialRes trial(const TrialIn &t) { return trial_warp<RP, CAT, EIG>(c, sm, ring, lane, t); }
  __device__ bool aborted() const { return false; }
};

// MINB: resident one-warp CTAs per SM the register allocation aims for
// (8: 255 registers per thread; 12: 168).
template <int RP, bool CAT = false, int EIG = 0, int MINB = kWarpTrialMinCtas>
__global__ void __launch_bounds__(32, MINB) k_place_warp(TrialCtx c, PlaceCtx p) {
  extern __shared__ __align__(16) char t_smem[];
  TrialSmem sm;
  float4 *ring;
  warp_trial_setup(c, t_smem, sm, ring, !(CAT && EIG));
  WarpTeam<RP, CAT, EIG> tm{c, sm, ring, (int)(threadIdx.x & 31)};
  place_queries(tm, c, p);
}

// A team of the tensor-core kernel (128 threads, its own named barrier,
// mbarrier and TMEM columns): thread 0 leads, the team's barrier orders, a
// shared int broadcasts.
struct TcTeam {
  const TrialCtx &c;
  const TcSmem &sm;
  uint32_t tmem;
  uint32_t &phase;
  bool &failed;
  int tid;
  __device__ bool leader() const { return tid == 0; }
  __device__ void sync() const { pgb::tc::team_sync(sm.bar_id); }
  __device__ int bcast(int v) const {
    pgb::tc::team_sync(sm.bar_id);  // earlier readers of the slot are done
    if (tid == 0) *sm.redi = v;
    pgb::tc::team_sync(sm.bar_id);
    return *sm.redi;
  }
  __device__ TrialRes trial(const TrialIn &t) { return tc_trial(c, sm, tmem, phase, failed, t, tid); }
  __device__ bool aborted() const { return failed; }
};

// The CTA of the CUDA-core trial kernel as a team (CAT models and the
// other CTA-tuned cases).
template <int K, int T, bool QNG = false>
struct CtaTeam {
  const TrialCtx &c;
  const TrialSmem &sm;
  __device__ bool leader() const { return threadIdx.x == 0; }
  __device__ void sync() const { __syncthreads(); }
  __device__ int bcast(int v) const {
    __syncthreads();  // earlier readers of the slot are done
    if (threadIdx.x == 0) *sm.redi = v;
    __syncthreads();
    return *sm.redi;
  }
  __device__ TrialRes trial(const TrialIn &t) { return trial_cta<K, T, QNG>(c, sm, t); }
  __device__ bool aborted() const { return false; }
};

template <int K, int T, bool QNG = false>
__global__ void __launch_bounds__(T, 1) k_place_cta(TrialCtx c, PlaceCtx p) {
  extern __shared__ __align__(16) char t_smem[];
  const TrialSmem sm = carve(t_smem, c.cap, c.smem_win, c.RP, K, c.NM, c.ncode);
  trial_cta_setup<K, T>(c, sm);
  CtaTeam<K, T, QNG> tm{c, sm};
  place_queries(tm, c, p);
}

// Whole queries on the tensor-core trial kernel (20-state Gamma mixtures):
// blockDim.x / 128 teams per CTA, each running the shared search on its own
// queries, with each trial run by the team; the teams share the CTA's
// constant B tiles and split its 512 TMEM columns.
__global__ void __launch_bounds__(kTcThreads * kTcMaxTeams, 1) k_place_tc(TrialCtx c, PlaceCtx p) {
  extern __shared__ __align__(16) char t_smem[];
  const int teams = blockDim.x / kTcThreads;
  const int team = threadIdx.x / kTcThreads, tid = threadIdx.x - team * kTcThreads;
  const TcSmem sm = tc_carve(t_smem, c.cap, c.NM, c.ncode, c.zcodes, team);
  const uint32_t tmem = tc_setup(c, sm, threadIdx.x, blockDim.x, teams) + kTcTeamCols * (uint32_t)team;
  uint32_t phase = 0;
  bool failed = false;
  TcTeam tm{c, sm, tmem, phase, failed, tid};
  place_queries(tm, c, p);
  tc_teardown(sm, phase, failed, threadIdx.x, teams);
}

}  // namespace
}  // namespace pgb

// ---------------------------------------------------------------------------
// Engine object
// ---------------------------------------------------------------------------
using namespace pgb;

struct pgb_engine {
  int K = 4, NM = 1, gcat = 0, S = 0, n_nodes = 0, root = -1, n_edges = 0, RP = 1, ncode = 18, prim = 4;
  int device = 0, n_sm = 0;
  size_t smem_optin = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev[8] = {};
  cudaStream_t bin_st[8] = {};   // the trial bins run concurrently, one stream each
  cudaEvent_t bin_ev[9] = {};
  std::vector<double> statd, X, lam, Xit, rates;
  std::vector<int> site_cats, parent, ch_start, ch_list, edge_nodes;
  std::vector<double> bl;
  // device model / tree
  double *d_bl = nullptr, *d_Xd = nullptr, *d_Xitd = nullptr, *d_lamd = nullptr, *d_ratesd = nullptr,
         *d_statdd = nullptr, *d_lvd = nullptr, *d_pm = nullptr, *d_pmh = nullptr;
  float *d_mf = nullptr;  // X, W, Lt, lvf, statd, lam, rates (float)
  size_t off_X = 0, off_W = 0, off_Lt = 0, off_lv = 0, off_statd = 0, off_lam = 0, off_rates = 0, off_Xit = 0;
  uint8_t *d_site_cat = nullptr, *d_char_code = nullptr, *d_informative = nullptr;
  uint16_t *d_col_order = nullptr;  // CAT: columns grouped by category (query site order)
  int *d_edge_nodes = nullptr, *d_parent = nullptr, *d_ch_start = nullptr, *d_ch_list = nullptr;
  // GLVs
  float *d_darr = nullptr, *d_parr = nullptr, *d_snode = nullptr;
  // darr / parr in the eigenbasis of the rate matrix (rows X^-1 v), for the
  // tensor-core trial kernel; built on first use after the GLVs change
  float *d_darr_e = nullptr, *d_parr_e = nullptr;
  bool eig_ready = false;
  // nucleotide eigenbasis warp form: the rate matrix has one zero eigenvalue
  // whose eigenvector (a column of X) is constant; eig_ord packs its index
  // (byte 0) and the other three (bytes 1..3), eig_c0 that column's value
  bool eig_ok = false;
  int eig_ord = 0;
  double eig_c0 = 0.0;
  int warp_variant = 0;  // the nucleotide Gamma warp form (launch_place_warp_gmix)
  int *d_dexp = nullptr, *d_pexp = nullptr, *d_sexp = nullptr;
  bool glvs_ready = false;
  // stage 1: edge tables (bf16 MMA operands, TMA descriptors), per-site
  // query classes, ambiguity list
  int Sp = 0;                       // sites padded to a multiple of 8 (table row pitch)
  int Sc = 0;                       // sites padded to a multiple of 32 (query class row pitch)
  float *d_qe = nullptr;
  __nv_bfloat16 *d_B3 = nullptr, *d_BX = nullptr;
  int *d_ebase = nullptr, *d_s1_err = nullptr;
  CUtensorMap tmT, tmX;
  uint8_t *d_qc = nullptr;
  size_t qc_cap = 0;
  bool s1_attr = false;
  // kernel launch shapes, set and queried once: the largest dynamic shared
  // memory set per kernel, and resident CTAs per SM per (kernel, threads, bytes)
  struct KernelSmem { const void *kern; size_t smem; };
  struct KernelFit { const void *kern; int threads; size_t smem; int per_sm; };
  std::vector<KernelSmem> k_smem;
  std::vector<KernelFit> k_fit;
  // page-locked status block a run copies back once: the trial counters and
  // the tensor-core kernels' error records
  struct RunStatus { unsigned long long stats[4]; int s1_err[4]; int tc_err[16]; };
  RunStatus *h_run = nullptr;
  int *d_qamb = nullptr, *d_amb_list = nullptr;
  std::vector<int> h_qamb, h_amb;
  double lt_pend = -1;
  // queries
  int Q = 0, Qcap = 0;
  char *d_seqs = nullptr;
  uint8_t *d_qcode = nullptr, *d_mcode = nullptr;
  uint16_t *d_reind = nullptr;
  uint32_t *d_rcode = nullptr;  // (alignment column << 8) | code per informative site
  int *d_qlen = nullptr, *d_qstatus = nullptr;
  std::vector<int> h_qlen;
  std::vector<int> h_len_at;  // counting-sort bins of the whole-query order (longest first)
  int *h_qinfo = nullptr;       // page-locked [3][Q]: lengths, ambiguity counts, the query order
  size_t h_qinfo_cap = 0;
  // run buffers
  double *d_scores = nullptr;  // FP64 stage-1 rows of queries with ambiguity characters (or all, on request)
  size_t scores_cap = 0;
  int2 *d_pairs = nullptr;     // tensor-core stage-1 pairs (C, exponent sum) [Q][n_edges]
  size_t pairs_cap = 0;
  int *d_plain_list = nullptr;
  size_t plain_cap = 0;
  int s1_nq = 0;               // the last stage-1 launch's query tile width
  int *d_rank = nullptr;
  size_t rank_cap = 0;
  BBState *d_bb = nullptr;
  ResEntry *d_res = nullptr;
  size_t res_cap = 0;
  size_t run_qcap = 0, run_kcap = 0;  // per-query run buffers (d_bb .. d_out) and the kept-placement slots
  int *d_tbase = nullptr, *d_tcount = nullptr, *d_keep_idx = nullptr, *d_keep_n = nullptr;
  TrialIn *d_trials = nullptr;
  TrialRes *d_tres = nullptr;
  int *d_bin_list = nullptr;
  size_t trials_cap = 0;
  unsigned long long *d_stats = nullptr;  // trial-kernel evaluation counters
  int *d_tc_err = nullptr;  // set by the tensor-core trial kernel when a completion wait timed out
  int *d_small = nullptr;  // counters: [0] trial counter, [1] n_active, [2..2+bins) bin counts, then bin limits
  pgb_placement *d_out = nullptr;
  int *d_qorder = nullptr;  // queries longest first (whole-query warp kernel)
  size_t qorder_cap = 0;
  double *d_gl = nullptr;        // Gauss-Legendre rule of the marginal likelihood
  double *d_prior_mu = nullptr;  // pendant prior mean per node, for (mu_prior, mu_lower)
  std::vector<double> h_prior_mu;
  int mu_prior = -1;
  double mu_lower = 0;
  int *d_nout = nullptr;
  int out_keep = 0;
  // trial-kernel shape per length bin: threads per CTA, shared-memory windows
  // allowed (1) or read from L2 (0); set by pgb_engine_autotune
  int tune_threads[8] = {256, 256, 256, 256, 256, 256, 256, 256};
  int tune_win[8] = {1, 1, 1, 1, 1, 1, 1, 1};
  // timings
  double t_ms[6] = {0, 0, 0, 0, 0, 0};
  double counts[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace pgb {
namespace {
// A kernel's dynamic shared-memory limit, raised (never lowered) to smem
// once per engine, so a placement run's launches make no attribute calls.
pgb_status kernel_smem(pgb_engine *e, const void *kern, size_t smem) {
  for (auto &k : e->k_smem)
    if (k.kern == kern) {
      if (k.smem >= smem) return PGB_OK;
      PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k.smem = smem;
      return PGB_OK;
    }
  PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  e->k_smem.push_back({kern, smem});
  return PGB_OK;
}

// kernel_smem plus the resident CTAs per SM at that launch shape (cached).
pgb_status kernel_fit(pgb_engine *e, const void *kern, int threads, size_t smem, int *per_sm) {
  pgb_status s;
  if ((s = kernel_smem(e, kern, smem))) return s;
  for (const auto &f : e->k_fit)
    if (f.kern == kern && f.threads == threads && f.smem == smem) { *per_sm = f.per_sm; return PGB_OK; }
  int n = 0;
  PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem));
  e->k_fit.push_back({kern, threads, smem, n});
  *per_sm = n;
  return PGB_OK;
}

}  // namespace
}  // namespace pgb

namespace {

constexpr int kBins = 6;
constexpr int kTuneTc = 1;  // tuning code of the tensor-core trial kernel

template <class T>
pgb_status dalloc(T **p, size_t n) {
  if (*p) { cudaFree(*p); *p = nullptr; }
  if (n == 0) n = 1;
  PGB_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
  return PGB_OK;
}
template <class T>
pgb_status upload(T **p, const T *h, size_t n, cudaStream_t st) {
  pgb_status s = dalloc(p, n);
  if (s) return s;
  if (n) PGB_CUDA(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return PGB_OK;
}
int grid_for(long n, int threads = 256) {
  long b = (n + threads - 1) / threads;
  return (int)std::max(1L, std::min(b, 152L * 32));
}

// Host P(t) for each matrix index (diagd.ml:79-98) in FP64.
void host_pmats(const pgb_engine *e, double t, std::vector<double> &pm) {
  int K = e->K;
  pm.assign((size_t)e->NM * K * K, 0.0);
  for (int m = 0; m < e->NM; m++)
    for (int i = 0; i < K; i++)
      for (int j = 0; j < K; j++) {
        double acc = 0;
        for (int k = 0; k < K; k++) acc += exp(e->rates[m] * t * e->lam[k]) * e->X[i * K + k] * e->Xit[j * K + k];
        pm[((size_t)m * K + i) * K + j] = acc;
      }
}

pgb_status ensure_queries(pgb_engine *e, int Q) {
  if (Q <= e->Qcap) return PGB_OK;
  size_t n = (size_t)Q * e->S;
  pgb_status s;
  if ((s = dalloc(&e->d_seqs, n)) || (s = dalloc(&e->d_qcode, n)) || (s = dalloc(&e->d_mcode, n)) ||
      (s = dalloc(&e->d_reind, n)) || (s = dalloc(&e->d_rcode, n)) || (s = dalloc(&e->d_qlen, Q)) ||
      (s = dalloc(&e->d_qstatus, Q)) ||
      (s = dalloc(&e->d_qamb, Q)) || (s = dalloc(&e->d_amb_list, Q)))
    return s;
  e->Qcap = Q;
  return PGB_OK;
}

S1Ctx stage1_ctx(pgb_engine *e) {
  S1Ctx c{};
  c.S = e->S; c.Sp = e->Sp; c.RP = e->RP; c.K = e->K; c.NM = e->NM; c.gcat = e->gcat; c.ncode = e->ncode;
  c.prim = e->prim; c.n_edges = e->n_edges; c.snode = e->d_snode; c.sexp = e->d_sexp;
  c.edge_nodes = e->d_edge_nodes; c.qe = e->d_qe; c.site_cat = e->d_site_cat;
  return c;
}

typedef CUresult (*TensorMapEncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                           const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                           CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                           CUtensorMapFloatOOBfill);

// TMA descriptors of the stage-1 tables: boxes of 32 sites x 128 edges
// (x 1 code x 3 planes, or x 2 digits), 64-byte swizzle, zero fill past the
// last site and edge.
pgb_status encode_stage1_maps(pgb_engine *e) {
  static TensorMapEncodeTiledFn enc = nullptr;
  if (!enc) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      set_error("stage 1: cuTensorMapEncodeTiled entry point unavailable");
      return PGB_ERR_CUDA;
    }
    enc = reinterpret_cast<TensorMapEncodeTiledFn>(fn);
  }
  const cuuint64_t row = (cuuint64_t)e->Sp * 2;
  {
    cuuint64_t dim[4] = {(cuuint64_t)e->S, (cuuint64_t)e->n_edges, (cuuint64_t)e->prim, 3};
    cuuint64_t stride[3] = {row, row * e->n_edges, row * e->n_edges * e->prim};
    cuuint32_t box[4] = {s1::kSites, s1::kEdges, 1, 3}, es[4] = {1, 1, 1, 1};
    CUresult r = enc(&e->tmT, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, e->d_B3, dim, stride, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("stage 1: tensor map of the log tables (%d)", (int)r); return PGB_ERR_CUDA; }
  }
  {
    cuuint64_t dim[3] = {(cuuint64_t)e->S, (cuuint64_t)e->n_edges, 2};
    cuuint64_t stride[2] = {row, row * e->n_edges};
    cuuint32_t box[3] = {s1::kSites, s1::kEdges, 2}, es[3] = {1, 1, 1};
    CUresult r = enc(&e->tmX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, e->d_BX, dim, stride, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("stage 1: tensor map of the exponent digits (%d)", (int)r); return PGB_ERR_CUDA; }
  }
  return PGB_OK;
}

pgb_status build_stage1_table(pgb_engine *e, double start_pend) {
  if (e->d_B3 && e->lt_pend == start_pend) return PGB_OK;
  int K = e->K;
  std::vector<double> pm;
  host_pmats(e, start_pend, pm);
  std::vector<float> qe((size_t)e->NM * e->ncode * K);
  std::vector<double> lv(K);
  for (int m = 0; m < e->NM; m++)
    for (int c = 0; c < e->ncode; c++) {
      code_lv(K, c, lv.data());
      for (int k = 0; k < K; k++) {  // gemmish of the LV by P (linear_c.c:29-90)
        double acc = 0;
        for (int j = 0; j < K; j++) acc += pm[((size_t)m * K + k) * K + j] * lv[j];
        qe[((size_t)m * e->ncode + c) * K + k] = (float)acc;
      }
    }
  pgb_status s;
  if ((s = upload(&e->d_qe, qe.data(), qe.size(), e->st))) return s;
  const size_t plane = (size_t)e->prim * e->n_edges * e->Sp;
  if (!e->d_B3) {
    if ((s = dalloc(&e->d_B3, 3 * plane)) || (s = dalloc(&e->d_BX, 2 * (size_t)e->n_edges * e->Sp)) ||
        (s = dalloc(&e->d_ebase, e->n_edges)) || (s = dalloc(&e->d_s1_err, 8)))
      return s;
    if ((s = encode_stage1_maps(e))) return s;
  }
  PGB_CUDA(cudaMemsetAsync(e->d_s1_err, 0, 8 * sizeof(int), e->st));
  k_s1_tables<<<e->n_edges, 256, 0, e->st>>>(stage1_ctx(e), e->d_B3, e->d_BX, e->d_ebase, e->d_s1_err);
  PGB_LAUNCH_CHECK();
  int h = 0;
  PGB_CUDA(cudaMemcpyAsync(&h, e->d_s1_err, sizeof h, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  if (h) {
    set_error("stage 1: supernode exponents out of the exact range of the tensor-core sums "
              "(per-site deviation from the edge mean >= 2^15, digit sums >= 2^24, or mean x sites >= 2^30)");
    return PGB_ERR_ARG;
  }
  e->lt_pend = start_pend;
  return PGB_OK;
}

// Per-site classes of the loaded queries (the B operands of k_s1_mma) and
// the list of queries with ambiguity characters; once per query load.
pgb_status prep_stage1_queries(pgb_engine *e) {
  pgb_status s;
  // rows for any query tile width up to 256 (n_qtiles * nq < Q + 256)
  const int rows = (e->Q + s1::kQueries - 1) / s1::kQueries * s1::kQueries + s1::kQueries;
  const size_t n = (size_t)rows * e->Sc;
  if (n > e->qc_cap) {
    if ((s = dalloc(&e->d_qc, n))) return s;
    e->qc_cap = n;
  }
  s1::k_s1_qclass<<<rows, 128, 0, e->st>>>(e->Q, e->S, e->Sc, e->prim, e->d_qcode, e->d_informative, e->d_qstatus,
                                       e->d_qc);
  PGB_LAUNCH_CHECK();
  e->h_amb.clear();
  for (int q = 0; q < e->Q; q++)
    if (e->h_qamb[q] > 0) e->h_amb.push_back(q);
  if (!e->h_amb.empty())
    PGB_CUDA(cudaMemcpyAsync(e->d_amb_list, e->h_amb.data(), e->h_amb.size() * 4, cudaMemcpyHostToDevice, e->st));
  return PGB_OK;
}

// Query tile width of k_s1_mma: the multiple of 16 in [128, 256] whose
// waves over the SMs cost least.  A tile's table stream (TMA of the edge
// rows from L2) does not shrink with its width; measured on dna_1k shapes it
// weighs as ~450 query columns, so narrower tiles pay only when they save a
// wave on small launches.
int s1_tile_queries(const pgb_engine *e) {
  const long n_etiles = (e->n_edges + s1::kEdges - 1) / s1::kEdges;
  int best = s1::kQueries;
  double best_cost = 1e300;
  for (int nq = s1::kQueries; nq >= 128; nq -= 16) {
    const long tiles = n_etiles * ((e->Q + nq - 1) / nq);
    const long waves = (tiles + e->n_sm - 1) / e->n_sm;
    const double cost = (double)waves * (nq + 448);
    if (cost < best_cost - 1e-9) { best_cost = cost; best = nq; }
  }
  return best;
}

pgb_status launch_s1_scores(pgb_engine *e, int rows, const int *d_list, int ambig) {
  if (rows < 1) return PGB_OK;
  dim3 grid((unsigned)rows, (unsigned)((e->n_edges + 127) / 128));
  k_s1_scores<<<grid, 128, 0, e->st>>>(stage1_ctx(e), rows, d_list, ambig, e->d_reind, e->d_mcode, e->d_qlen,
                                       e->d_qstatus, e->d_pairs, e->gcat ? 0.0 : log((double)(float)e->NM),
                                       e->d_scores);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// Stage 1 on the loaded queries: the tensor-core pairs [Q][n_edges], and the
// FP64 score rows of the queries with ambiguity characters (all_scores:
// every query's FP64 row, for pgb_queries_stage1).
pgb_status run_stage1(pgb_engine *e, bool all_scores = false) {
  pgb_status s;
  const size_t qe_n = (size_t)e->Q * e->n_edges;
  if (qe_n > e->pairs_cap) {
    if ((s = dalloc(&e->d_pairs, qe_n))) return s;
    e->pairs_cap = qe_n;
  }
  if ((all_scores || !e->h_amb.empty()) && qe_n > e->scores_cap) {
    if ((s = dalloc(&e->d_scores, qe_n))) return s;
    e->scores_cap = qe_n;
  }
  if (e->Q < 1) return PGB_OK;
  s1::MmaCtx c{};
  c.S = e->S; c.n_chunks = e->Sc / s1::kSites; c.prim = e->prim; c.n_edges = e->n_edges; c.Q = e->Q;
  c.nq = s1_tile_queries(e);
  c.n_qtiles = (e->Q + c.nq - 1) / c.nq; c.Sc = e->Sc;
  c.qc = e->d_qc; c.qlen = e->d_qlen; c.qstatus = e->d_qstatus; c.ebase = e->d_ebase;
  c.pairs = e->d_pairs;
  c.err = e->d_s1_err;
  e->s1_nq = c.nq;
  if (!e->s1_attr) {  // per engine, and so per device
    PGB_CUDA(cudaFuncSetAttribute(s1::k_s1_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1::kSmemBytes));
    e->s1_attr = true;
  }
  const int n_etiles = (e->n_edges + s1::kEdges - 1) / s1::kEdges;
  s1::k_s1_mma<<<n_etiles * c.n_qtiles, s1::kThreads, s1::kSmemBytes, e->st>>>(e->tmT, e->tmX, c);
  PGB_LAUNCH_CHECK();
  if ((s = launch_s1_scores(e, (int)e->h_amb.size(), e->d_amb_list, 1))) return s;
  if (all_scores) {
    if ((size_t)e->Q > e->plain_cap) {
      if ((s = dalloc(&e->d_plain_list, e->Q))) return s;
      e->plain_cap = e->Q;
    }
    std::vector<int> plain;
    for (int q = 0; q < e->Q; q++)
      if (e->h_qamb[q] == 0) plain.push_back(q);
    if (!plain.empty()) {
      PGB_CUDA(cudaMemcpyAsync(e->d_plain_list, plain.data(), plain.size() * 4, cudaMemcpyHostToDevice, e->st));
      if ((s = launch_s1_scores(e, (int)plain.size(), e->d_plain_list, 0))) return s;
      PGB_CUDA(cudaStreamSynchronize(e->st));  // plain is a pageable host buffer
    }
  }
  return PGB_OK;
}

pgb_status run_rank(pgb_engine *e, int rk) {
  const int E = e->n_edges;
  const size_t keys = (size_t)E * 8;
  // up to 4 warps (queries) per block; keys staged (within 96 KB) only for
  // long rankings, where lanes refill their caches often
  int nw = 4, in_smem = rk > 16 * kRankCache ? 1 : 0;
  if (in_smem) {
    while (nw > 1 && nw * keys > 96 * 1024) nw--;
    if (nw * keys > e->smem_optin) in_smem = 0;
  }
  size_t smem = in_smem ? nw * keys : 0;
  if (smem > 48 * 1024) {
    pgb_status s = kernel_smem(e, (const void *)k_rank_warp, smem);
    if (s) return s;
  }
  S1Scores sv{e->d_pairs, e->d_scores, e->d_qlen, e->d_qamb, e->gcat ? 0.0 : log((double)(float)e->NM)};
  k_rank_warp<<<(e->Q + nw - 1) / nw, 32 * nw, smem, e->st>>>(sv, E, rk, e->Q, e->d_qstatus, e->d_rank,
                                                              in_smem);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// the character codes the query-vector tables of the warp and tensor-core
// kernels hold: the primary states, or every code when a loaded query has an
// ambiguity character
int tc_zcodes(const pgb_engine *e) {
  for (int a : e->h_qamb)
    if (a > 0) return e->ncode;
  return e->prim;
}

TrialCtx trial_ctx(pgb_engine *e, const pgb_prefs *p, int optimizer, int mode) {
  TrialCtx c{};
  c.darr = e->d_darr; c.parr = e->d_parr; c.dexp = e->d_dexp; c.pexp = e->d_pexp;
  c.S = e->S; c.RP = e->RP; c.K = e->K; c.NM = e->NM; c.ncode = e->ncode; c.gcat = e->gcat;
  c.bl = e->d_bl; c.reind = e->d_reind; c.mcode = e->d_mcode; c.rcode = e->d_rcode; c.qlen = e->d_qlen;
  c.site_cat = e->d_site_cat; c.qamb = e->d_qamb; c.prim = e->prim;
  c.X = e->d_mf + e->off_X; c.W = e->d_mf + e->off_W; c.Lt = e->d_mf + e->off_Lt; c.lvf = e->d_mf + e->off_lv;
  c.statd = e->d_mf + e->off_statd; c.lam = e->d_mf + e->off_lam; c.rates = e->d_mf + e->off_rates;
  c.Xit = e->d_mf + e->off_Xit;
  c.tc_err = e->d_tc_err;
  c.darr_e = e->d_darr_e; c.parr_e = e->d_parr_e;
  c.eig_ord = e->eig_ord;
  c.zcodes = tc_zcodes(e);
  c.log_nrates = e->gcat ? 0.0 : log((double)(float)e->NM);
  c.start_pend = p->start_pend;
  c.max_pend = p->max_pend;
  c.optimizer = optimizer;
  c.mode = mode;
  c.stats = e->d_stats;
  c.gl = e->d_gl;
  c.pp_rule = (p->calc_pp || mode == 2) ? p->pp_rule : 0;  // only marginal likelihoods use it
  c.pp_rel_err = p->pp_rel_err;
  return c;
}

// window capacities of the trial bins (sites); the last bin reads the
// windows from global memory
void bin_limits(const pgb_engine *e, int *lim) {
  static const int caps4[kBins] = {256, 512, 768, 1024, 1536, 1 << 30};
  for (int b = 0; b < kBins; b++) lim[b] = caps4[b];
  if (e->K != 4 || e->gcat) {  // wider sites: fewer smem-staged bins
    lim[0] = 128; lim[1] = 256; lim[2] = 384; lim[3] = 512; lim[4] = 640; lim[5] = 1 << 30;
  }
}

template <int K, int T, bool QNG = false>
pgb_status launch_trials_kt(pgb_engine *e, cudaStream_t st, TrialCtx c, const int *d_order, int n, int cap, bool win,
                            TrialRes *out) {
  c.smem_win = win ? 1 : 0;
  c.cap = cap;
  size_t smem = trial_smem_bytes(cap, c.smem_win, e->RP, K, e->NM, e->ncode);
  if (smem > e->smem_optin) { set_error("trial shared memory %zu exceeds %zu", smem, e->smem_optin); return PGB_ERR_ARG; }
  pgb_status s = kernel_smem(e, (const void *)k_trials<K, T, QNG>, smem);
  if (s) return s;
  k_trials<K, T, QNG><<<n, T, smem, st>>>(c, e->d_trials, d_order, n, out);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// the warp-per-trial kernel covers nucleotide Gamma mixtures of 1, 2, 4 or 8 rates
// the warp-per-trial kernel for per-site CAT models (one GLV plane), when
// the categories' tables fit the shared memory of a one-warp CTA
bool warp_cat_ok(const pgb_engine *e) {
  return e->K == 4 && e->gcat && e->RP == 1 && e->NM <= 255 &&
         warp_trial_smem_bytes(e->NM, e->ncode, e->ncode) <= e->smem_optin;
}

bool warp_trials_ok(const pgb_engine *e) {
  return e->K == 4 && !e->gcat && e->NM == e->RP && (e->RP == 1 || e->RP == 2 || e->RP == 4 || e->RP == 8);
}

// one warp per trial applies (Gamma mixtures or CAT)
bool warp_form_ok(const pgb_engine *e) { return warp_trials_ok(e) || warp_cat_ok(e); }

template <int RP, bool CAT = false>
pgb_status launch_trials_warp_rp(pgb_engine *e, cudaStream_t st, TrialCtx c, const WarpSegs &segs, TrialRes *out) {
  size_t smem = warp_trial_smem_bytes(e->NM, e->ncode, c.zcodes);
  if (smem > e->smem_optin) { set_error("warp trial shared memory %zu exceeds %zu", smem, e->smem_optin); return PGB_ERR_ARG; }
  pgb_status s = kernel_smem(e, (const void *)k_trials_warp<RP, CAT>, smem);
  if (s) return s;
  int grid = (segs.n + kWarpTrialWarps - 1) / kWarpTrialWarps;
  k_trials_warp<RP, CAT><<<grid, 32 * kWarpTrialWarps, smem, st>>>(c, e->d_trials, segs, out);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

pgb_status launch_trials_warp(pgb_engine *e, cudaStream_t st, TrialCtx c, const WarpSegs &segs, TrialRes *out) {
  if (segs.nseg < 1 || segs.n <= 0) return PGB_OK;
  c.smem_win = 0;
  c.cap = 0;
  if (e->gcat) return launch_trials_warp_rp<1, true>(e, st, c, segs, out);
  switch (e->RP) {
    case 1: return launch_trials_warp_rp<1>(e, st, c, segs, out);
    case 2: return launch_trials_warp_rp<2>(e, st, c, segs, out);
    case 4: return launch_trials_warp_rp<4>(e, st, c, segs, out);
    default: return launch_trials_warp_rp<8>(e, st, c, segs, out);
  }
}

// the tensor-core trial kernel covers 20-state Gamma mixtures of up to 4 rates
bool tc_trials_ok(const pgb_engine *e) { return e->K == kTcK && !e->gcat && e->NM == e->RP && e->RP <= kTcMaxRates; }

// the eigenbasis warp form applies (and is the one selected when `selected`)
bool warp_eig_ok(const pgb_engine *e) { return warp_trials_ok(e) && e->eig_ok; }

// darr / parr in eigen-coordinates, for the kernels that read them: the
// tensor-core kernel (20 states) and the eigenbasis warp form (nucleotides,
// the permuted and premultiplied layout of k_eigen_glvs_dna).
pgb_status ensure_eigen_glvs(pgb_engine *e) {
  const bool tc = tc_trials_ok(e),
             dna = (warp_eig_ok(e) && e->warp_variant != 0) || (warp_cat_ok(e) && e->eig_ok && e->warp_variant != 0);
  if (e->eig_ready || (!tc && !dna)) return PGB_OK;
  const long rows = (long)e->n_nodes * e->S * e->RP;
  pgb_status s;
  if (!e->d_darr_e && ((s = dalloc(&e->d_darr_e, (size_t)rows * e->K)) || (s = dalloc(&e->d_parr_e, (size_t)rows * e->K))))
    return s;
  if (tc)
    k_eigen_glvs<<<grid_for(2 * rows), 256, 0, e->st>>>(e->d_darr, e->d_parr, e->d_Xitd, rows, e->d_darr_e,
                                                        e->d_parr_e);
  else
    k_eigen_glvs_dna<<<grid_for(2 * rows), 256, 0, e->st>>>(e->d_darr, e->d_parr, e->d_Xitd, rows, e->eig_ord,
                                                            e->eig_c0, e->d_darr_e, e->d_parr_e);
  PGB_LAUNCH_CHECK();
  e->eig_ready = true;
  return PGB_OK;
}

// Dynamic shared memory of a tensor-core trial launch: at least enough that
// no more CTAs fit on an SM than its 512 TMEM columns serve (2 with one team
// of 256 columns each, 1 with two teams), so no CTA ever waits for columns.
size_t tc_launch_smem(pgb_engine *e, size_t smem, int teams) {
  int sm_smem = 0;
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->device);
  const size_t per_cta = (size_t)sm_smem / (teams == 1 ? 3 : 2) + 1024;
  return std::min(std::max(smem, per_cta), e->smem_optin);
}

pgb_status launch_trials_tc(pgb_engine *e, cudaStream_t st, TrialCtx c, const int *d_order, int n, int cap,
                            TrialRes *out) {
  c.smem_win = 0;
  c.cap = std::max(cap, 1);
  c.zcodes = tc_zcodes(e);
  size_t smem = tc_trial_smem_bytes(c.cap, e->NM, e->ncode, c.zcodes, 1);
  if (smem > e->smem_optin) { set_error("tensor-core trial shared memory %zu exceeds %zu", smem, e->smem_optin); return PGB_ERR_ARG; }
  smem = tc_launch_smem(e, smem, 1);
  pgb_status s = kernel_smem(e, (const void *)k_trials_tc, smem);
  if (s) return s;
  k_trials_tc<<<n, kTcThreads, smem, st>>>(c, e->d_trials, d_order, n, out);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// Error records of the tensor-core kernels (bounded waits that timed out),
// g: the stage-1 record, h: the trial kernels' record, both already on the
// host; a set record is cleared on the device and reported.
pgb_status report_tc_err(pgb_engine *e, const int *g, const int *h) {
  if (e->d_s1_err && g[0]) {
    PGB_CUDA(cudaMemsetAsync(e->d_s1_err, 0, 4 * sizeof(int), e->st));
    set_error("stage-1 tensor-core kernel: a pipeline wait timed out (role %d, unit %d, block %d)", g[1], g[2], g[3]);
    return PGB_ERR_CUDA;
  }
  if (h[0]) {
    PGB_CUDA(cudaMemsetAsync(e->d_tc_err, 0, 16 * sizeof(int), e->st));
    set_error("tensor-core trial kernel: an MMA completion wait timed out (cta %d rate %d chunk %d phase %d: "
              "wait %d test %d/%d; tmem 0x%x, tiles 0x%x, barrier 0x%x; sites %d chunks %d)",
              h[1], h[2], h[3], h[4], h[5], h[6], h[7], h[8], h[9], h[10], h[11], h[12]);
    return PGB_ERR_CUDA;
  }
  return PGB_OK;
}

// the same, reading the records from the device
pgb_status check_tc_err(pgb_engine *e) {
  if (e->d_s1_err) {
    int g[4];
    PGB_CUDA(cudaMemcpy(g, e->d_s1_err, sizeof g, cudaMemcpyDeviceToHost));
    if (g[0]) {
      PGB_CUDA(cudaMemsetAsync(e->d_s1_err, 0, sizeof g, e->st));
      set_error("stage-1 tensor-core kernel: a pipeline wait timed out (role %d, unit %d, block %d)", g[1], g[2],
                g[3]);
      return PGB_ERR_CUDA;
    }
  }
  int h[16];
  PGB_CUDA(cudaMemcpy(h, e->d_tc_err, sizeof h, cudaMemcpyDeviceToHost));
  if (h[0]) {
    PGB_CUDA(cudaMemsetAsync(e->d_tc_err, 0, sizeof h, e->st));
    set_error("tensor-core trial kernel: an MMA completion wait timed out (cta %d rate %d chunk %d phase %d: "
              "wait %d test %d/%d; tmem 0x%x, tiles 0x%x, barrier 0x%x; sites %d chunks %d)",
              h[1], h[2], h[3], h[4], h[5], h[6], h[7], h[8], h[9], h[10], h[11], h[12]);
    return PGB_ERR_CUDA;
  }
  return PGB_OK;
}

// threads: 32 selects the warp-per-trial kernel where it applies, 1 the
// tensor-core CTA kernel where it applies, else the CTA-per-trial kernel with
// 128 or 256 threads
pgb_status launch_trials(pgb_engine *e, cudaStream_t st, TrialCtx c, const int *d_order, int n, int cap, bool win,
                         TrialRes *out, int threads) {
  if (n <= 0) return PGB_OK;
  if (c.pp_rule == 1) {  // the reference's marginal likelihood: only the CTA kernels built with it carry it
    if (threads != 128) threads = 256;
    if (threads == 256 && trial_smem_bytes(cap, win, e->RP, e->K, e->NM, e->ncode) > e->smem_optin) win = false;
    if (e->K == 4)
      return threads == 128 ? launch_trials_kt<4, 128, true>(e, st, c, d_order, n, cap, win, out)
                            : launch_trials_kt<4, 256, true>(e, st, c, d_order, n, cap, win, out);
    return threads == 128 ? launch_trials_kt<20, 128, true>(e, st, c, d_order, n, cap, win, out)
                          : launch_trials_kt<20, 256, true>(e, st, c, d_order, n, cap, win, out);
  }
  if (threads == kTuneTc) {
    if (tc_trials_ok(e)) return launch_trials_tc(e, st, c, d_order, n, cap, out);
    threads = 256;
  }
  if (threads == 32) {
    if (warp_form_ok(e)) {
      WarpSegs segs{};
      segs.list[0] = d_order;
      segs.start[0] = 0;
      segs.start[1] = n;
      segs.nseg = 1;
      segs.n = n;
      return launch_trials_warp(e, st, c, segs, out);
    }
    threads = 256;
  }
  if (e->K == 4)
    return threads == 128 ? launch_trials_kt<4, 128>(e, st, c, d_order, n, cap, win, out)
                          : launch_trials_kt<4, 256>(e, st, c, d_order, n, cap, win, out);
  return threads == 128 ? launch_trials_kt<20, 128>(e, st, c, d_order, n, cap, win, out)
                        : launch_trials_kt<20, 256>(e, st, c, d_order, n, cap, win, out);
}

// window capacity of bin b and whether it is staged in shared memory
void bin_shape(const pgb_engine *e, int b, int max_sq, int allow_win, int *cap, bool *win) {
  int lim[kBins];
  bin_limits(e, lim);
  size_t win_budget = e->smem_optin - trial_smem_bytes(0, 0, e->RP, e->K, e->NM, e->ncode) - 2048;
  int c0 = std::min(lim[b], max_sq);
  *win = allow_win && b < kBins - 1 && (size_t)2 * e->RP * c0 * e->K * 4 + 2 * (size_t)c0 <= win_budget;
  *cap = *win ? std::max(c0, 1) : std::max(max_sq, 1);
}

// Launch every non-empty bin of the trial lists, concurrently (one stream
// each, longest windows first), and join them on the engine stream.
pgb_status run_bins(pgb_engine *e, TrialCtx c, const int *h_bin_count, int max_sq) {
  bool all_warp = warp_form_ok(e) && c.pp_rule != 1;  // the QNG replica runs on the CTA kernels
  for (int b = 0; b < kBins; b++)
    if (h_bin_count[b] > 0 && e->tune_threads[b] != 32) all_warp = false;
  if (all_warp) {  // one launch over every bin, longest bin first
    WarpSegs segs{};
    int tot = 0;
    for (int b = kBins - 1; b >= 0; b--) {
      if (h_bin_count[b] == 0) continue;
      segs.list[segs.nseg] = e->d_bin_list + (long)b * e->trials_cap;
      segs.start[segs.nseg] = tot;
      tot += h_bin_count[b];
      segs.nseg++;
    }
    segs.start[segs.nseg] = tot;
    segs.n = tot;
    return launch_trials_warp(e, e->st, c, segs, e->d_tres);
  }
  PGB_CUDA(cudaEventRecord(e->bin_ev[8], e->st));
  int used[kBins], nu = 0;
  for (int b = kBins - 1; b >= 0; b--) {
    int n = h_bin_count[b];
    if (n == 0) continue;
    int cap;
    bool win;
    bin_shape(e, b, max_sq, e->tune_win[b], &cap, &win);
    cudaStream_t bs = e->bin_st[b];
    PGB_CUDA(cudaStreamWaitEvent(bs, e->bin_ev[8], 0));
    pgb_status s = launch_trials(e, bs, c, e->d_bin_list + (long)b * e->trials_cap, n, cap, win, e->d_tres,
                                 e->tune_threads[b]);
    if (s) return s;
    PGB_CUDA(cudaEventRecord(e->bin_ev[b], bs));
    used[nu++] = b;
  }
  for (int i = 0; i < nu; i++) PGB_CUDA(cudaStreamWaitEvent(e->st, e->bin_ev[used[i]], 0));
  return PGB_OK;
}

pgb_status ensure_run_buffers(pgb_engine *e, const pgb_prefs *p, int rk, int maxr, size_t tcap) {
  pgb_status s;
  size_t rn = (size_t)e->Q * rk;
  if (rn > e->rank_cap) { if ((s = dalloc(&e->d_rank, rn))) return s; e->rank_cap = rn; }
  size_t resn = (size_t)e->Q * maxr;
  if (resn > e->res_cap) { if ((s = dalloc(&e->d_res, resn))) return s; e->res_cap = resn; }
  // per-query run buffers: reallocated only when the query count or
  // keep_at_most outgrows them (a reallocation synchronises the device)
  if ((size_t)e->Q > e->run_qcap || (size_t)e->Q * p->keep_at_most > e->run_kcap) {
    const size_t nq = std::max((size_t)e->Q, e->run_qcap), nk = std::max((size_t)e->Q * p->keep_at_most, e->run_kcap);
    if ((s = dalloc(&e->d_bb, nq)) || (s = dalloc(&e->d_tbase, nq)) || (s = dalloc(&e->d_tcount, nq)) ||
        (s = dalloc(&e->d_keep_n, nq)) || (s = dalloc(&e->d_keep_idx, nk)) || (s = dalloc(&e->d_nout, nq)) ||
        (s = dalloc(&e->d_out, nk))) {
      e->run_qcap = e->run_kcap = 0;
      return s;
    }
    e->run_qcap = nq;
    e->run_kcap = nk;
  }
  if (tcap > e->trials_cap) {
    if ((s = dalloc(&e->d_trials, tcap)) || (s = dalloc(&e->d_tres, tcap)) ||
        (s = dalloc(&e->d_bin_list, tcap * kBins)))
      return s;
    e->trials_cap = tcap;
  }
  e->out_keep = p->keep_at_most;
  return PGB_OK;
}

// Gauss-Legendre rule on [-1, 1]: the roots of P_n by Newton's method from
// the Chebyshev-like guess cos(pi (i + 3/4) / (n + 1/2)), P_n and P_n' by the
// three-term recurrence; weights 2 / ((1 - x^2) P_n'(x)^2).
void gauss_legendre(int n, double *x, double *w) {
  for (int i = 0; i < n; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1;
    for (int it = 0; it < 100; it++) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= n; k++) {
        double pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = n * (z * p1 - p0) / (z * z - 1);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = -z;  // ascending
    w[i] = 2 / ((1 - z * z) * dp * dp);
  }
}

// Pendant prior means per node (pplacer_run.ml:379-389): the flat
// exponential's mean is the tree length over the edge count; the informative
// prior's mean at node i is the average over the leaves below i of their
// distance to i, plus bl(i) + prior_lower (core.ml:34-51, top_segment_f =
// (+) prior_lower).
pgb_status ensure_prior_means(pgb_engine *e, int prior, double prior_lower) {
  if (e->d_prior_mu && e->mu_prior == prior && e->mu_lower == prior_lower) return PGB_OK;
  std::vector<double> mu(e->n_nodes, 0.0);
  if (prior == 2) {
    std::vector<double> cnt(e->n_nodes, 0.0), sum(e->n_nodes, 0.0);
    for (int i = 0; i < e->n_nodes; i++) {  // post-order: children before parents
      if (e->ch_start[i + 1] == e->ch_start[i]) cnt[i] = 1;
      mu[i] = sum[i] / cnt[i] + e->bl[i] + prior_lower;
      int p = e->parent[i];
      if (p >= 0) { cnt[p] += cnt[i]; sum[p] += sum[i] + cnt[i] * e->bl[i]; }
    }
  } else {
    double len = 0;
    for (int i : e->edge_nodes) len += e->bl[i];
    for (double &m : mu) m = len / e->n_edges;
  }
  pgb_status s;
  if ((s = upload(&e->d_prior_mu, mu.data(), mu.size(), e->st))) return s;
  e->h_prior_mu = mu;
  e->mu_prior = prior;
  e->mu_lower = prior_lower;
  return PGB_OK;
}

template <int RP, bool CAT = false, int EIG = 0, int MINB = kWarpTrialMinCtas>
pgb_status launch_place_warp_rp(pgb_engine *e, TrialCtx c, const PlaceCtx &pc) {
  size_t smem = warp_trial_smem_bytes(e->NM, e->ncode, c.zcodes, !(CAT && EIG));
  auto kern = k_place_warp<RP, CAT, EIG, MINB>;
  int per_sm = 0;
  pgb_status s = kernel_fit(e, (const void *)kern, 32, smem, &per_sm);
  if (s) return s;
  int grid = std::max(1, std::min(e->Q, e->n_sm * std::max(1, per_sm)));
  kern<<<grid, 32, smem, e->st>>>(c, pc);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// The nucleotide Gamma warp forms (the autotuner's choice, warp_variant):
// 0 matrices in registers, 8 warps per SM; 1, 2, 3 eigenbasis at 8, 12 and
// 16 warps per SM (255, 168 and 128 registers); 4, 5 the eigenbasis on
// packed FP32 pairs at 12 and 16 warps per SM.
constexpr int kWarpForms = 6;
// The CAT warp forms: 0 matrices per category, 1 the eigenbasis, 2 the
// eigenbasis on packed FP32 pairs.
constexpr int kCatForms = 3;
constexpr int kCatEigMinCtas = 12;  // the CAT eigenbasis form: one-warp CTAs per SM it aims for
template <int RP>
pgb_status launch_place_warp_gmix(pgb_engine *e, TrialCtx c, const PlaceCtx &pc) {
  if (e->warp_variant == 1) return launch_place_warp_rp<RP, false, 1, 8>(e, c, pc);
  if (e->warp_variant == 2) return launch_place_warp_rp<RP, false, 1, 12>(e, c, pc);
  if (e->warp_variant == 3) return launch_place_warp_rp<RP, false, 1, 16>(e, c, pc);
  if (e->warp_variant == 4) return launch_place_warp_rp<RP, false, 2, 12>(e, c, pc);
  if (e->warp_variant == 5) return launch_place_warp_rp<RP, false, 2, 16>(e, c, pc);
  return launch_place_warp_rp<RP>(e, c, pc);
}

pgb_status launch_place_tc(pgb_engine *e, TrialCtx c, const PlaceCtx &pc, int max_sq) {
  c.cap = std::max(max_sq, 1);
  c.zcodes = tc_zcodes(e);
  // Two teams per CTA when the shared memory holds them (they share the B
  // tiles and split the SM's TMEM columns), else one; one persistent CTA per
  // SM, the teams taking queries from the shared counter.
  int teams = kTcMaxTeams;
  size_t smem = tc_trial_smem_bytes(c.cap, e->NM, e->ncode, c.zcodes, teams);
  if (smem > e->smem_optin) {
    teams = 1;
    smem = tc_trial_smem_bytes(c.cap, e->NM, e->ncode, c.zcodes, teams);
  }
  if (smem > e->smem_optin) { set_error("tensor-core trial shared memory %zu exceeds %zu", smem, e->smem_optin); return PGB_ERR_ARG; }
  smem = tc_launch_smem(e, smem, teams);
  pgb_status s = kernel_smem(e, (const void *)k_place_tc, smem);
  if (s) return s;
  const int grid = std::max(1, std::min((e->Q + teams - 1) / teams, e->n_sm));
  k_place_tc<<<grid, kTcThreads * teams, smem, e->st>>>(c, pc);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

template <int K, int T, bool QNG = false>
pgb_status launch_place_cta_kt(pgb_engine *e, TrialCtx c, const PlaceCtx &pc, int max_sq, int win) {
  int cap = std::max(max_sq, 1);
  size_t smem = trial_smem_bytes(cap, win, e->RP, K, e->NM, e->ncode);
  if (win && smem > e->smem_optin) {  // the windows do not fit: read them from L2
    win = 0;
    smem = trial_smem_bytes(cap, 0, e->RP, K, e->NM, e->ncode);
  }
  if (smem > e->smem_optin) { set_error("trial shared memory %zu exceeds %zu", smem, e->smem_optin); return PGB_ERR_ARG; }
  c.cap = cap;
  c.smem_win = win;
  int per_sm = 0;
  pgb_status s = kernel_fit(e, (const void *)k_place_cta<K, T, QNG>, T, smem, &per_sm);
  if (s) return s;
  int grid = std::max(1, std::min(e->Q, e->n_sm * std::max(1, per_sm)));
  k_place_cta<K, T, QNG><<<grid, T, smem, e->st>>>(c, pc);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

// the CTA form of whole queries, with the bins' common tuning
pgb_status launch_place_cta(pgb_engine *e, TrialCtx c, const PlaceCtx &pc, int max_sq) {
  const int T = e->tune_threads[0], win = e->tune_win[0];
  if (c.pp_rule == 1) {  // the reference's marginal likelihood: the CTA kernels built with it
    if (e->K == 4)
      return T == 128 ? launch_place_cta_kt<4, 128, true>(e, c, pc, max_sq, win)
                      : launch_place_cta_kt<4, 256, true>(e, c, pc, max_sq, T == 256 ? win : 0);
    return T == 128 ? launch_place_cta_kt<20, 128, true>(e, c, pc, max_sq, win)
                    : launch_place_cta_kt<20, 256, true>(e, c, pc, max_sq, T == 256 ? win : 0);
  }
  if (e->K == 4)
    return T == 128 ? launch_place_cta_kt<4, 128>(e, c, pc, max_sq, win)
                    : launch_place_cta_kt<4, 256>(e, c, pc, max_sq, win);
  return T == 128 ? launch_place_cta_kt<20, 128>(e, c, pc, max_sq, win)
                  : launch_place_cta_kt<20, 256>(e, c, pc, max_sq, win);
}

// whole queries in one persistent launch: every bin tuned to the same form
// (the warp form for nucleotide Gamma mixtures, the tensor-core form for 20
// states, or one CTA size; the CTA form stages the windows when the first
// bin does and the longest query's fit)
bool whole_query_form(const pgb_engine *e) {
  for (int b = 1; b < kBins; b++)
    if (e->tune_threads[b] != e->tune_threads[0]) return false;
  const int t = e->tune_threads[0];
  if (t == 32) return warp_form_ok(e);
  if (t == kTuneTc) return tc_trials_ok(e);
  return t == 128 || t == 256;
}

// Stage 2 and refinement as one persistent launch of whole-query warps (or
// whole-query CTAs: tensor-core for 20-state models, CUDA-core otherwise).
pgb_status run_whole_queries(pgb_engine *e, const pgb_prefs *p, const BBCtx &c, TrialCtx tc, int max_sq) {
  pgb_status s;
  PGB_CUDA(cudaMemsetAsync(e->d_small, 0, sizeof(int), e->st));
  tc.smem_win = 0;
  tc.cap = 0;
  PlaceCtx pc{};
  pc.bb = c;
  pc.qorder = e->d_qorder;
  pc.qnext = e->d_small;
  pc.keep_at_most = p->keep_at_most;
  pc.log_keep_factor = log(p->keep_factor);
  pc.out = e->d_out;
  pc.n_out = e->d_nout;
  pc.tstats = e->d_stats + 2;
  pc.calc_pp = p->calc_pp;
  pc.prior_kind = p->prior == 1 ? 0 : 1;
  if ((s = ensure_prior_means(e, p->prior, p->prior_lower))) return s;
  pc.prior_mu = e->d_prior_mu;
  if (tc.pp_rule == 1) s = launch_place_cta(e, tc, pc, max_sq);  // the CTA kernels carry the QNG replica
  else if (e->tune_threads[0] == kTuneTc && tc_trials_ok(e)) s = launch_place_tc(e, tc, pc, max_sq);
  else if (e->tune_threads[0] != 32 || !warp_form_ok(e)) s = launch_place_cta(e, tc, pc, max_sq);
  else if (e->gcat)  // the CAT forms: 0 matrices per category, 1 the eigenbasis, 2 on packed FP32 pairs
    s = e->warp_variant == 1 && e->eig_ok   ? launch_place_warp_rp<1, true, 1, kCatEigMinCtas>(e, tc, pc)
        : e->warp_variant == 2 && e->eig_ok ? launch_place_warp_rp<1, true, 2, kCatEigMinCtas>(e, tc, pc)
                                            : launch_place_warp_rp<1, true>(e, tc, pc);
  else
    switch (e->RP) {
      case 1: s = launch_place_warp_gmix<1>(e, tc, pc); break;
      case 2: s = launch_place_warp_gmix<2>(e, tc, pc); break;
      case 4: s = launch_place_warp_gmix<4>(e, tc, pc); break;
      default: s = launch_place_warp_gmix<8>(e, tc, pc); break;
    }
  if (s) return s;
  PGB_CUDA(cudaEventRecord(e->ev[3], e->st));
  PGB_CUDA(cudaEventRecord(e->ev[4], e->st));
  // the counters and error records in one page-locked block, one wait
  pgb_engine::RunStatus *hr = e->h_run;
  PGB_CUDA(cudaMemcpyAsync(hr->stats, e->d_stats, sizeof hr->stats, cudaMemcpyDeviceToHost, e->st));
  if (e->d_s1_err) PGB_CUDA(cudaMemcpyAsync(hr->s1_err, e->d_s1_err, sizeof hr->s1_err, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaMemcpyAsync(hr->tc_err, e->d_tc_err, sizeof hr->tc_err, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  float ms;
  cudaEventElapsedTime(&ms, e->ev[1], e->ev[5]); e->t_ms[0] = ms;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]); e->t_ms[1] = ms;
  cudaEventElapsedTime(&ms, e->ev[1], e->ev[2]); e->t_ms[2] = ms;
  cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]); e->t_ms[3] = ms;
  e->t_ms[4] = 0;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[4]); e->t_ms[5] = ms;
  const unsigned long long *st_h = hr->stats;
  if ((s = report_tc_err(e, hr->s1_err, hr->tc_err))) return s;
  e->counts[1] = (double)(st_h[2] + st_h[3]);
  e->counts[2] = (double)st_h[0];
  e->counts[3] = (double)st_h[1];
  e->counts[4] = e->counts[5] = (double)st_h[2];
  e->counts[6] = (double)st_h[3];
  e->counts[7] = 1;
  return PGB_OK;
}

}  // namespace

extern "C" {

void pgb_prefs_default(pgb_prefs *p) {
  p->start_pend = 0.1;
  p->max_pend = 2.0;
  p->initial_tolerance = 0.01;
  p->max_strikes = 6;
  p->strike_box = 3.0;
  p->max_pitches = 40;
  p->keep_at_most = 7;
  p->keep_factor = 0.01;
  p->optimizer = 1;
  p->calc_pp = 0;
  p->prior = 0;
  p->pp_rel_err = 0.01;
  p->prior_lower = 0.0;
  p->pp_rule = 0;
}

static pgb_status prep_queries(pgb_engine *e);

// CAT models: the alignment columns sorted by (category, column) -- the
// order in which k_query_prep lists a query's sites
static pgb_status upload_col_order(pgb_engine *e) {
  if (!e->gcat) return PGB_OK;
  std::vector<uint16_t> ord(e->S);
  for (int i = 0; i < e->S; i++) ord[i] = (uint16_t)i;
  std::stable_sort(ord.begin(), ord.end(), [&](uint16_t a, uint16_t b) { return e->site_cats[a] < e->site_cats[b]; });
  if (!e->d_col_order) {
    pgb_status s = dalloc(&e->d_col_order, (size_t)e->S);
    if (s) return s;
  }
  PGB_CUDA(cudaMemcpyAsync(e->d_col_order, ord.data(), (size_t)e->S * sizeof(uint16_t), cudaMemcpyHostToDevice,
                           e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));  // before the host vector goes
  return PGB_OK;
}

pgb_status pgb_engine_create(const pgb_model_desc *m, const pgb_tree_desc *t, pgb_engine **out) {
  if (!m || !t || !out) { set_error("engine_create: null argument"); return PGB_ERR_ARG; }
  if ((m->n_states != 4 && m->n_states != 20) || m->n_rates < 1 || m->n_rates > 64 || m->n_sites < 1 ||
      m->n_sites > 65535 || t->n_nodes < 2) {
    set_error("engine_create: unsupported sizes (n_states 4|20, n_rates 1..64, n_sites 1..65535)");
    return PGB_ERR_ARG;
  }
  if (m->gcat && !m->site_categories) { set_error("engine_create: gcat needs site_categories"); return PGB_ERR_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    set_error("engine_create: no CUDA device");
    return PGB_ERR_CUDA;
  }
  pgb_engine *e = new pgb_engine();
  e->K = m->n_states;
  e->NM = m->n_rates;
  e->gcat = m->gcat ? 1 : 0;
  e->RP = e->gcat ? 1 : e->NM;
  e->S = m->n_sites;
  e->ncode = n_codes(e->K);
  e->prim = e->K;
  e->Sp = (e->S + 7) & ~7;
  e->Sc = (e->S + s1::kSites - 1) / s1::kSites * s1::kSites;
  int K = e->K;
  e->statd.assign(m->statd, m->statd + K);
  e->X.assign(m->x, m->x + K * K);
  e->lam.assign(m->lambda, m->lambda + K);
  e->Xit.assign(m->xit, m->xit + K * K);
  e->rates.assign(m->rates, m->rates + e->NM);
  if (K == 4) {  // the eigenbasis warp form needs one zero eigenvalue with a constant eigenvector
    int kz = 0;
    double lmax = 0;
    for (int k = 0; k < K; k++) {
      lmax = std::max(lmax, std::fabs(e->lam[k]));
      if (e->lam[k] > e->lam[kz]) kz = k;
    }
    bool ok = lmax > 0 && std::fabs(e->lam[kz]) <= 1e-9 * lmax;
    for (int k = 0; k < K && ok; k++)
      if (k != kz && std::fabs(e->lam[k]) <= 1e-6 * lmax) ok = false;
    const double c0 = e->X[kz];
    for (int i = 0; i < K && ok; i++)
      if (!(std::fabs(e->X[i * K + kz] - c0) <= 1e-9 * std::fabs(c0))) ok = false;
    if (ok) {
      int ord = kz, s = 1;
      for (int k = 0; k < K; k++)
        if (k != kz) ord |= k << (8 * s++);
      e->eig_ok = true;
      e->eig_ord = ord;
      // until the autotuner says otherwise: the eigenbasis form on packed FP32
      // pairs at 12 warps per SM (Gamma mixtures), the CAT eigenbasis form on
      // packed FP32 pairs
      e->warp_variant = e->gcat ? 2 : 4;
      double mean = 0;
      for (int i = 0; i < K; i++) mean += e->X[i * K + kz];
      e->eig_c0 = mean / K;
    }
  }
  if (e->gcat) {
    e->site_cats.assign(m->site_categories, m->site_categories + e->S);
    for (int v : e->site_cats)
      if (v < 0 || v >= e->NM) { set_error("engine_create: site category out of range"); delete e; return PGB_ERR_ARG; }
  }
  e->n_nodes = t->n_nodes;
  e->parent.assign(t->parent, t->parent + t->n_nodes);
  e->bl.assign(t->bl, t->bl + t->n_nodes);
  std::vector<std::vector<int>> ch(e->n_nodes);
  for (int i = 0; i < e->n_nodes; i++) {
    int p = e->parent[i];
    if (p < 0) {
      if (e->root >= 0) { set_error("engine_create: more than one root"); delete e; return PGB_ERR_ARG; }
      e->root = i;
    } else if (p <= i || p >= e->n_nodes) {
      set_error("engine_create: nodes must be numbered post-order (parent id > child id)");
      delete e;
      return PGB_ERR_ARG;
    } else ch[p].push_back(i);
  }
  if (e->root < 0) { set_error("engine_create: no root"); delete e; return PGB_ERR_ARG; }
  e->bl[e->root] = 0.0;
  e->ch_start.assign(e->n_nodes + 1, 0);
  for (int i = 0; i < e->n_nodes; i++) {
    e->ch_start[i + 1] = e->ch_start[i] + (int)ch[i].size();
    for (int c : ch[i]) e->ch_list.push_back(c);
    if (i != e->root) e->edge_nodes.push_back(i);
  }
  if (e->ch_list.empty()) e->ch_list.push_back(0);
  e->n_edges = (int)e->edge_nodes.size();

  cudaError_t ce;
  if ((ce = cudaGetDevice(&e->device)) != cudaSuccess || (ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking)) != cudaSuccess) {
    set_error("engine_create: %s", cudaGetErrorString(ce));
    delete e;
    return PGB_ERR_CUDA;
  }
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device);
  cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
  e->smem_optin = (size_t)optin;
  if (warp_form_ok(e))  // one warp per trial unless the autotuner finds better
    for (int b = 0; b < kBins; b++) { e->tune_threads[b] = 32; e->tune_win[b] = 0; }
  if (tc_trials_ok(e))  // tensor-core CTAs unless the autotuner finds better
    for (int b = 0; b < kBins; b++) { e->tune_threads[b] = kTuneTc; e->tune_win[b] = 0; }
  for (int i = 0; i < 8; i++) cudaEventCreate(&e->ev[i]);
  if ((ce = cudaHostAlloc((void **)&e->h_run, sizeof(pgb_engine::RunStatus), cudaHostAllocDefault)) != cudaSuccess) {
    set_error("engine_create: %s", cudaGetErrorString(ce));
    delete e;
    return PGB_ERR_CUDA;
  }
  memset(e->h_run, 0, sizeof(pgb_engine::RunStatus));
  for (int i = 0; i < 8; i++) cudaStreamCreateWithFlags(&e->bin_st[i], cudaStreamNonBlocking);
  for (int i = 0; i < 9; i++) cudaEventCreateWithFlags(&e->bin_ev[i], cudaEventDisableTiming);

  // model constants
  std::vector<float> mf;
  auto put = [&](const std::vector<float> &v) { size_t o = mf.size(); mf.insert(mf.end(), v.begin(), v.end()); while (mf.size() % 4) mf.push_back(0.f); return o; };
  std::vector<float> Xf(K * K), Xitf(K * K), W((size_t)K * K * K), Lt((size_t)e->ncode * K), lvf((size_t)e->ncode * K), sf(K), lf(K),
      rf(e->NM);
  std::vector<double> lvd((size_t)e->ncode * K), lv(K);
  for (int i = 0; i < K * K; i++) { Xf[i] = (float)e->X[i]; Xitf[i] = (float)e->Xit[i]; }
  for (int i = 0; i < K; i++)
    for (int j = 0; j < K; j++)
      for (int k = 0; k < K; k++) W[((size_t)i * K + j) * K + k] = (float)(e->X[i * K + k] * e->Xit[j * K + k]);
  for (int c = 0; c < e->ncode; c++) {
    code_lv(K, c, lv.data());
    for (int k = 0; k < K; k++) {
      double acc = 0;
      for (int j = 0; j < K; j++) acc += e->Xit[j * K + k] * lv[j];
      Lt[(size_t)c * K + k] = (float)acc;
      lvf[(size_t)c * K + k] = (float)lv[k];
      lvd[(size_t)c * K + k] = lv[k];
    }
  }
  for (int i = 0; i < K; i++) { sf[i] = (float)e->statd[i]; lf[i] = (float)e->lam[i]; }
  for (int i = 0; i < e->NM; i++) rf[i] = (float)e->rates[i];
  e->off_X = put(Xf); e->off_W = put(W); e->off_Lt = put(Lt); e->off_lv = put(lvf);
  e->off_statd = put(sf); e->off_lam = put(lf); e->off_rates = put(rf); e->off_Xit = put(Xitf);
  // character tables
  std::vector<uint8_t> cc(256, kBadCode), inf(kMaxCodes, 0);
  const char *alpha = code_alphabet(K);
  for (int c = 0; c < e->ncode; c++) {
    cc[(uint8_t)alpha[c]] = (uint8_t)c;
    inf[c] = code_informative(K, c) ? 1 : 0;
  }
  std::vector<uint8_t> scat(e->S, 0);
  if (e->gcat)
    for (int s = 0; s < e->S; s++) scat[s] = (uint8_t)e->site_cats[s];
  std::vector<double> glr(2 * kGlPoints);
  gauss_legendre(kGlPoints, glr.data(), glr.data() + kGlPoints);
  pgb_status s;
  if ((s = upload(&e->d_mf, mf.data(), mf.size(), e->st)) || (s = upload(&e->d_bl, e->bl.data(), e->bl.size(), e->st)) ||
      (s = upload(&e->d_Xd, e->X.data(), e->X.size(), e->st)) ||
      (s = upload(&e->d_Xitd, e->Xit.data(), e->Xit.size(), e->st)) ||
      (s = upload(&e->d_lamd, e->lam.data(), e->lam.size(), e->st)) ||
      (s = upload(&e->d_ratesd, e->rates.data(), e->rates.size(), e->st)) ||
      (s = upload(&e->d_statdd, e->statd.data(), e->statd.size(), e->st)) ||
      (s = upload(&e->d_lvd, lvd.data(), lvd.size(), e->st)) ||
      (s = upload(&e->d_gl, glr.data(), glr.size(), e->st)) ||
      (s = upload(&e->d_site_cat, scat.data(), scat.size(), e->st)) ||
      (s = upload_col_order(e)) ||
      (s = upload(&e->d_char_code, cc.data(), cc.size(), e->st)) ||
      (s = upload(&e->d_informative, inf.data(), inf.size(), e->st)) ||
      (s = upload(&e->d_edge_nodes, e->edge_nodes.data(), e->edge_nodes.size(), e->st)) ||
      (s = upload(&e->d_parent, e->parent.data(), e->parent.size(), e->st)) ||
      (s = upload(&e->d_ch_start, e->ch_start.data(), e->ch_start.size(), e->st)) ||
      (s = upload(&e->d_ch_list, e->ch_list.data(), e->ch_list.size(), e->st)) ||
      (s = dalloc(&e->d_small, 64)) || (s = dalloc(&e->d_stats, 4)) || (s = dalloc(&e->d_tc_err, 16))) {
    pgb_engine_destroy(e);
    return s;
  }
  if ((ce = cudaMemsetAsync(e->d_tc_err, 0, 16 * sizeof(int), e->st)) != cudaSuccess) {
    set_error("engine_create: %s", cudaGetErrorString(ce));
    pgb_engine_destroy(e);
    return PGB_ERR_CUDA;
  }
  // P matrices of every node at bl and bl/2 (FP64)
  size_t npm = (size_t)e->n_nodes * e->NM * K * K;
  if ((s = dalloc(&e->d_pm, npm)) || (s = dalloc(&e->d_pmh, npm))) { pgb_engine_destroy(e); return s; }
  k_node_pmats<<<grid_for((long)npm), 256, 0, e->st>>>(e->d_pm, e->d_bl, 1.0, e->n_nodes, e->NM, K, e->d_Xd,
                                                       e->d_Xitd, e->d_lamd, e->d_ratesd);
  count_launch();
  k_node_pmats<<<grid_for((long)npm), 256, 0, e->st>>>(e->d_pmh, e->d_bl, 0.5, e->n_nodes, e->NM, K, e->d_Xd,
                                                       e->d_Xitd, e->d_lamd, e->d_ratesd);
  count_launch();
  if (cudaStreamSynchronize(e->st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    set_error("engine_create: setup kernels failed");
    pgb_engine_destroy(e);
    return PGB_ERR_CUDA;
  }
  *out = e;
  return PGB_OK;
}

pgb_status pgb_engine_destroy(pgb_engine *e) {
  if (!e) return PGB_OK;
  if (e->st) cudaStreamSynchronize(e->st);
  if (e->h_run) cudaFreeHost(e->h_run);
  if (e->h_qinfo) cudaFreeHost(e->h_qinfo);
  void *ptrs[] = {e->d_bl, e->d_Xd, e->d_Xitd, e->d_lamd, e->d_ratesd, e->d_statdd, e->d_lvd, e->d_pm, e->d_pmh,
                  e->d_mf, e->d_site_cat, e->d_char_code, e->d_informative, e->d_edge_nodes, e->d_parent,
                  e->d_ch_start, e->d_ch_list, e->d_darr, e->d_parr, e->d_snode, e->d_dexp, e->d_pexp, e->d_sexp,
                  e->d_qe, e->d_B3, e->d_BX, e->d_ebase, e->d_s1_err, e->d_qc, e->d_qamb,
                  e->d_amb_list, e->d_seqs, e->d_qcode, e->d_mcode, e->d_reind, e->d_rcode, e->d_qlen,
                  e->d_qstatus, e->d_scores, e->d_pairs, e->d_plain_list, e->d_rank, e->d_bb, e->d_res, e->d_tbase, e->d_tcount, e->d_keep_idx, e->d_keep_n,
                  e->d_trials, e->d_tres, e->d_bin_list, e->d_small, e->d_out, e->d_nout, e->d_stats,
                  e->d_qorder, e->d_gl, e->d_prior_mu, e->d_darr_e, e->d_parr_e, e->d_tc_err,
                  e->d_col_order};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int i = 0; i < 8; i++)
    if (e->ev[i]) cudaEventDestroy(e->ev[i]);
  for (int i = 0; i < 8; i++)
    if (e->bin_st[i]) cudaStreamDestroy(e->bin_st[i]);
  for (int i = 0; i < 9; i++)
    if (e->bin_ev[i]) cudaEventDestroy(e->bin_ev[i]);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
  return PGB_OK;
}

static pgb_status alloc_glv_store(pgb_engine *e) {
  size_t n = (size_t)e->n_nodes * e->S * e->RP * e->K, ne = (size_t)e->n_nodes * e->S;
  pgb_status s;
  if ((s = dalloc(&e->d_darr, n)) || (s = dalloc(&e->d_parr, n)) || (s = dalloc(&e->d_snode, n)) ||
      (s = dalloc(&e->d_dexp, ne)) || (s = dalloc(&e->d_pexp, ne)) || (s = dalloc(&e->d_sexp, ne)))
    return s;
  e->lt_pend = -1;
  return PGB_OK;
}

// Leaves with their character codes, and the post-order (height) and
// pre-order (depth) levels of the tree passes.
struct TreeLevels {
  std::vector<int> leaves, hlist, hstart, dlist, dstart;
  std::vector<uint8_t> codes;
  int maxh = 0, maxd = 0;
};

pgb_status tree_levels(const pgb_engine *e, const int *leaf_row, const char *seqs, int n_rows, TreeLevels &t) {
  int K = e->K, S = e->S;
  const char *alpha = code_alphabet(K);
  for (int i = 0; i < e->n_nodes; i++) {
    if (e->ch_start[i + 1] != e->ch_start[i]) continue;
    int row = leaf_row[i];
    if (row < 0 || row >= n_rows) { set_error("precompute: leaf %d has no alignment row", i); return PGB_ERR_ARG; }
    t.leaves.push_back(i);
    for (int s = 0; s < S; s++) {
      const char *p = strchr(alpha, seqs[(size_t)row * S + s]);
      if (!p || !seqs[(size_t)row * S + s]) { set_error("precompute: unknown character in reference row %d", row); return PGB_ERR_ARG; }
      t.codes.push_back((uint8_t)(p - alpha));
    }
  }
  std::vector<int> height(e->n_nodes, 0), depth(e->n_nodes, 0);
  for (int i = 0; i < e->n_nodes; i++)
    for (int c = e->ch_start[i]; c < e->ch_start[i + 1]; c++) height[i] = std::max(height[i], height[e->ch_list[c]] + 1);
  for (int i = e->n_nodes - 1; i >= 0; i--)
    if (e->parent[i] >= 0) depth[i] = depth[e->parent[i]] + 1;
  for (int i = 0; i < e->n_nodes; i++) { t.maxh = std::max(t.maxh, height[i]); t.maxd = std::max(t.maxd, depth[i]); }
  t.hstart.assign(t.maxh + 2, 0);
  t.dstart.assign(t.maxd + 2, 0);
  for (int h = 1; h <= t.maxh; h++) {
    t.hstart[h] = (int)t.hlist.size();
    for (int i = 0; i < e->n_nodes; i++) if (height[i] == h) t.hlist.push_back(i);
  }
  t.hstart[t.maxh + 1] = (int)t.hlist.size();
  for (int d = 1; d <= t.maxd; d++) {
    t.dstart[d] = (int)t.dlist.size();
    for (int i = 0; i < e->n_nodes; i++) if (depth[i] == d) t.dlist.push_back(i);
  }
  t.dstart[t.maxd + 1] = (int)t.dlist.size();
  return PGB_OK;
}

pgb_status pgb_engine_precompute(pgb_engine *e, const int *leaf_row, const char *seqs, int n_rows) {
  if (!e || !leaf_row || !seqs || n_rows < 1) { set_error("precompute: bad argument"); return PGB_ERR_ARG; }
  int K = e->K, S = e->S;
  TreeLevels tl;
  {
    pgb_status st = tree_levels(e, leaf_row, seqs, n_rows, tl);
    if (st) return st;
  }
  const std::vector<int> &leaves = tl.leaves, &hlist = tl.hlist, &hstart = tl.hstart, &dlist = tl.dlist,
                         &dstart = tl.dstart;
  const std::vector<uint8_t> &codes = tl.codes;
  const int maxh = tl.maxh, maxd = tl.maxd;
  size_t n = (size_t)e->n_nodes * S * e->RP * K, ne = (size_t)e->n_nodes * S;
  double *d_distal = nullptr, *d_evd = nullptr, *d_prox = nullptr;
  int *d_de = nullptr, *d_ee = nullptr, *d_pe = nullptr, *d_leaves = nullptr, *d_hlist = nullptr, *d_dlist = nullptr;
  uint8_t *d_codes = nullptr;
  pgb_status s = PGB_OK;
  auto cleanup = [&]() {
    void *ps[] = {d_distal, d_evd, d_prox, d_de, d_ee, d_pe, d_leaves, d_hlist, d_dlist, d_codes};
    for (void *p : ps) if (p) cudaFree(p);
  };
  if ((s = dalloc(&d_distal, n)) || (s = dalloc(&d_evd, n)) || (s = dalloc(&d_prox, n)) || (s = dalloc(&d_de, ne)) ||
      (s = dalloc(&d_ee, ne)) || (s = dalloc(&d_pe, ne)) ||
      (s = upload(&d_leaves, leaves.data(), leaves.size(), e->st)) ||
      (s = upload(&d_codes, codes.data(), codes.size(), e->st)) ||
      (s = upload(&d_hlist, hlist.data(), hlist.size(), e->st)) ||
      (s = upload(&d_dlist, dlist.data(), dlist.size(), e->st)) || (s = alloc_glv_store(e))) {
    cleanup();
    return s;
  }
  PreCtx c{};
  c.S = S; c.RP = e->RP; c.K = K; c.NM = e->NM; c.gcat = e->gcat; c.site_cat = e->d_site_cat; c.lvd = e->d_lvd;
  c.pm = e->d_pm; c.pmh = e->d_pmh; c.statd = e->d_statdd; c.distal = d_distal; c.evd = d_evd; c.prox = d_prox;
  c.de = d_de; c.ee = d_ee; c.pe = d_pe;
  k_leaves<<<grid_for((long)leaves.size() * S), 256, 0, e->st>>>(c, d_leaves, (int)leaves.size(), d_codes);
  count_launch();
  for (int h = 1; h <= maxh; h++) {
    int cnt = hstart[h + 1] - hstart[h];
    if (!cnt) continue;
    k_distal_level<<<grid_for((long)cnt * S), 256, 0, e->st>>>(c, d_hlist + hstart[h], cnt, e->d_ch_start,
                                                               e->d_ch_list);
    count_launch();
  }
  size_t root_off = (size_t)e->root * S * e->RP * K;
  k_set_unit<<<grid_for((long)S * e->RP * K), 256, 0, e->st>>>(d_prox + root_off, d_pe + (size_t)e->root * S,
                                                               (long)S * e->RP * K, (long)S);
  count_launch();
  for (int d = 1; d <= maxd; d++) {
    int cnt = dstart[d + 1] - dstart[d];
    if (!cnt) continue;
    k_prox_level<<<grid_for((long)cnt * S), 256, 0, e->st>>>(c, d_dlist + dstart[d], cnt, e->d_parent,
                                                             e->d_ch_start, e->d_ch_list);
    count_launch();
  }
  k_finish_glvs<<<grid_for((long)e->n_nodes * S), 256, 0, e->st>>>(c, e->n_nodes, e->d_darr, e->d_parr, e->d_snode,
                                                                   e->d_dexp, e->d_pexp, e->d_sexp);
  count_launch();
  cudaError_t ce = cudaStreamSynchronize(e->st);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  cleanup();
  if (ce != cudaSuccess) { set_error("precompute: %s", cudaGetErrorString(ce)); return PGB_ERR_CUDA; }
  e->glvs_ready = true;
  e->eig_ready = false;
  return PGB_OK;
}

pgb_status pgb_engine_refine_categories(pgb_engine *e, const int *leaf_row, const char *seqs, int n_rows,
                                        int *categories) {
  if (!e || !leaf_row || !seqs || n_rows < 1) { set_error("refine: bad argument"); return PGB_ERR_ARG; }
  if (!e->gcat) { set_error("refine: only per-site category models have site categories"); return PGB_ERR_STATE; }
  const int K = e->K, S = e->S;
  TreeLevels tl;
  pgb_status s = tree_levels(e, leaf_row, seqs, n_rows, tl);
  if (s) return s;
  size_t n = (size_t)e->n_nodes * S * K, ne = (size_t)e->n_nodes * S;
  double *d_distal = nullptr, *d_evd = nullptr, *d_best = nullptr;
  int *d_de = nullptr, *d_ee = nullptr, *d_leaves = nullptr, *d_hlist = nullptr, *d_bcat = nullptr;
  uint8_t *d_codes = nullptr;
  auto cleanup = [&]() {
    void *ps[] = {d_distal, d_evd, d_best, d_de, d_ee, d_leaves, d_hlist, d_bcat, d_codes};
    for (void *p : ps) if (p) cudaFree(p);
  };
  if ((s = dalloc(&d_distal, n)) || (s = dalloc(&d_evd, n)) || (s = dalloc(&d_de, ne)) || (s = dalloc(&d_ee, ne)) ||
      (s = dalloc(&d_best, S)) || (s = dalloc(&d_bcat, S)) ||
      (s = upload(&d_leaves, tl.leaves.data(), tl.leaves.size(), e->st)) ||
      (s = upload(&d_codes, tl.codes.data(), tl.codes.size(), e->st)) ||
      (s = upload(&d_hlist, tl.hlist.data(), tl.hlist.size(), e->st))) {
    cleanup();
    return s;
  }
  PreCtx c{};
  c.S = S; c.RP = 1; c.K = K; c.NM = e->NM; c.gcat = 1; c.site_cat = e->d_site_cat; c.lvd = e->d_lvd;
  c.pm = e->d_pm; c.pmh = e->d_pmh; c.statd = e->d_statdd; c.distal = d_distal; c.evd = d_evd;
  c.de = d_de; c.ee = d_ee;
  k_refine_init<<<grid_for(S), 256, 0, e->st>>>(d_best, d_bcat, S);
  count_launch();
  for (int cat = 0; cat < e->NM; cat++) {  // every site in category cat
    cudaError_t ce = cudaMemsetAsync(e->d_site_cat, cat, S, e->st);
    if (ce != cudaSuccess) { cleanup(); set_error("refine: %s", cudaGetErrorString(ce)); return PGB_ERR_CUDA; }
    k_leaves<<<grid_for((long)tl.leaves.size() * S), 256, 0, e->st>>>(c, d_leaves, (int)tl.leaves.size(), d_codes);
    count_launch();
    for (int h = 1; h <= tl.maxh; h++) {
      int cnt = tl.hstart[h + 1] - tl.hstart[h];
      if (!cnt) continue;
      k_distal_level<<<grid_for((long)cnt * S), 256, 0, e->st>>>(c, d_hlist + tl.hstart[h], cnt, e->d_ch_start,
                                                                 e->d_ch_list);
      count_launch();
    }
    double r = e->rates[cat];
    k_refine_site<<<grid_for(S), 256, 0, e->st>>>(d_distal + (size_t)e->root * S * K, d_de + (size_t)e->root * S,
                                                  e->d_statdd, S, K, cat, 2.0 * log(r) - 3.0 * r, d_best, d_bcat);
    count_launch();
  }
  std::vector<int> best(S);
  cudaError_t ce = cudaMemcpyAsync(best.data(), d_bcat, S * sizeof(int), cudaMemcpyDeviceToHost, e->st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
  cleanup();
  if (ce != cudaSuccess) { set_error("refine: %s", cudaGetErrorString(ce)); return PGB_ERR_CUDA; }
  for (int i = 0; i < S; i++)
    if (best[i] < 0) {  // gcat_model.ml:363-364
      set_error("refine: site %d has zero likelihood", i);
      return PGB_ERR_ARG;
    }
  e->site_cats = best;
  std::vector<uint8_t> sc(S);
  for (int i = 0; i < S; i++) sc[i] = (uint8_t)best[i];
  PGB_CUDA(cudaMemcpyAsync(e->d_site_cat, sc.data(), S, cudaMemcpyHostToDevice, e->st));
  pgb_status us = upload_col_order(e);  // the site lists follow the new categories
  if (!us) us = prep_queries(e);
  if (!us && e->Q > 0) us = prep_stage1_queries(e);
  if (us) return us;
  PGB_CUDA(cudaStreamSynchronize(e->st));
  e->glvs_ready = false;  // the placement GLVs follow the categories: precompute again
  e->eig_ready = false;
  e->lt_pend = -1;
  if (categories) std::copy(best.begin(), best.end(), categories);
  return PGB_OK;
}

pgb_status pgb_engine_set_glvs(pgb_engine *e, const double *darr, const int *darr_e, const double *parr,
                               const int *parr_e, const double *snodes, const int *snodes_e) {
  if (!e || !darr || !darr_e || !parr || !parr_e) { set_error("set_glvs: bad argument"); return PGB_ERR_ARG; }
  size_t n = (size_t)e->n_nodes * e->RP * e->S * e->K, ne = (size_t)e->n_nodes * e->S;
  pgb_status s = alloc_glv_store(e);
  if (s) return s;
  double *dd = nullptr, *dp = nullptr;
  int *ed = nullptr, *ep = nullptr;
  if ((s = upload(&dd, darr, n, e->st)) || (s = upload(&ed, darr_e, ne, e->st)) || (s = upload(&dp, parr, n, e->st)) ||
      (s = upload(&ep, parr_e, ne, e->st))) {
    cudaFree(dd); cudaFree(dp); cudaFree(ed); cudaFree(ep);
    return s;
  }
  k_import_glv<<<grid_for((long)n), 256, 0, e->st>>>(dd, ed, e->d_darr, e->d_dexp, e->n_nodes, e->S, e->RP, e->K);
  count_launch();
  k_import_glv<<<grid_for((long)n), 256, 0, e->st>>>(dp, ep, e->d_parr, e->d_pexp, e->n_nodes, e->S, e->RP, e->K);
  count_launch();
  if (snodes && snodes_e) {
    double *ds = nullptr;
    int *es = nullptr;
    if ((s = upload(&ds, snodes, n, e->st)) || (s = upload(&es, snodes_e, ne, e->st))) { cudaFree(ds); cudaFree(es); return s; }
    k_import_glv<<<grid_for((long)n), 256, 0, e->st>>>(ds, es, e->d_snode, e->d_sexp, e->n_nodes, e->S, e->RP, e->K);
    count_launch();
    cudaStreamSynchronize(e->st);
    cudaFree(ds);
    cudaFree(es);
  } else {
    k_snodes_from<<<grid_for((long)ne), 256, 0, e->st>>>(dd, dp, ed, ep, e->d_pmh, e->d_statdd, e->d_site_cat,
                                                         e->gcat, e->d_snode, e->d_sexp, e->n_nodes, e->S, e->RP,
                                                         e->K, e->NM);
    count_launch();
  }
  cudaError_t ce = cudaStreamSynchronize(e->st);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  cudaFree(dd); cudaFree(dp); cudaFree(ed); cudaFree(ep);
  if (ce != cudaSuccess) { set_error("set_glvs: %s", cudaGetErrorString(ce)); return PGB_ERR_CUDA; }
  e->glvs_ready = true;
  e->eig_ready = false;
  return PGB_OK;
}

pgb_status pgb_engine_get_glv(pgb_engine *e, int which, int node, double *a, int *ex) {
  if (!e || !e->glvs_ready || node < 0 || node >= e->n_nodes || which < 0 || which > 2) {
    set_error("get_glv: bad argument or no GLVs");
    return PGB_ERR_ARG;
  }
  size_t per = (size_t)e->S * e->RP * e->K;
  std::vector<float> buf(per);
  const float *src = which == 0 ? e->d_darr : which == 1 ? e->d_parr : e->d_snode;
  const int *esrc = which == 0 ? e->d_dexp : which == 1 ? e->d_pexp : e->d_sexp;
  PGB_CUDA(cudaMemcpyAsync(buf.data(), src + per * node, per * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaMemcpyAsync(ex, esrc + (size_t)e->S * node, (size_t)e->S * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  for (int s = 0; s < e->S; s++)
    for (int r = 0; r < e->RP; r++)
      for (int k = 0; k < e->K; k++)
        a[((size_t)r * e->S + s) * e->K + k] = buf[((size_t)s * e->RP + r) * e->K + k];
  return PGB_OK;
}

// the per-query site lists of the loaded sequences (d_seqs), in the order and
// with the categories of the current model
static pgb_status prep_queries(pgb_engine *e) {
  if (e->Q < 1) return PGB_OK;
  k_query_prep<<<e->Q, 256, 0, e->st>>>(e->d_seqs, e->S, e->prim, e->d_char_code, e->d_informative,
                                        e->gcat ? e->d_col_order : nullptr, e->gcat ? e->d_site_cat : nullptr,
                                        e->d_qcode, e->d_reind, e->d_mcode, e->d_rcode, e->d_qlen, e->d_qstatus,
                                        e->d_qamb);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}

pgb_status pgb_queries_load(pgb_engine *e, int n_queries, const char *seqs) {
  if (!e || n_queries < 0 || (n_queries > 0 && !seqs)) { set_error("queries_load: bad argument"); return PGB_ERR_ARG; }
  pgb_status s = ensure_queries(e, std::max(n_queries, 1));
  if (s) return s;
  e->Q = n_queries;
  if (!n_queries) return PGB_OK;
  PGB_CUDA(cudaMemcpyAsync(e->d_seqs, seqs, (size_t)n_queries * e->S, cudaMemcpyHostToDevice, e->st));
  if ((s = prep_queries(e))) return s;
  // lengths and ambiguity counts back through a page-locked staging block
  if ((size_t)n_queries > e->h_qinfo_cap) {
    PGB_CUDA(cudaStreamSynchronize(e->st));  // the previous load's order upload reads the old block
    if (e->h_qinfo) cudaFreeHost(e->h_qinfo);
    e->h_qinfo = nullptr;
    e->h_qinfo_cap = 0;
    PGB_CUDA(cudaHostAlloc((void **)&e->h_qinfo, (size_t)n_queries * 3 * sizeof(int), cudaHostAllocDefault));
    e->h_qinfo_cap = n_queries;
  }
  int *hq = e->h_qinfo;
  PGB_CUDA(cudaMemcpyAsync(hq, e->d_qlen, (size_t)n_queries * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaMemcpyAsync(hq + n_queries, e->d_qamb, (size_t)n_queries * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  e->h_qlen.assign(hq, hq + n_queries);
  e->h_qamb.assign(hq + n_queries, hq + 2 * n_queries);
  // the whole-query kernels take queries longest first from this order
  if ((size_t)n_queries > e->qorder_cap) {
    if ((s = dalloc(&e->d_qorder, n_queries))) return s;
    e->qorder_cap = n_queries;
  }
  // longest first, equal lengths in query order: a counting sort over the
  // lengths 0..S (O(Q + S) on the host, between two launches)
  std::vector<int> &at = e->h_len_at;
  int *ord = hq + 2 * n_queries;  // page-locked: the copy below runs asynchronously
  at.assign(e->S + 2, 0);
  for (int q = 0; q < n_queries; q++) at[e->S - e->h_qlen[q] + 1]++;
  for (int l = 1; l <= e->S + 1; l++) at[l] += at[l - 1];
  for (int q = 0; q < n_queries; q++) ord[at[e->S - e->h_qlen[q]]++] = q;
  PGB_CUDA(cudaMemcpyAsync(e->d_qorder, ord, (size_t)n_queries * sizeof(int), cudaMemcpyHostToDevice, e->st));
  return prep_stage1_queries(e);
}

static pgb_status check_prefs(const pgb_prefs *p) {
  if (!p || p->keep_at_most < 1 || p->keep_at_most > 64 || p->max_pitches < 0 || p->max_strikes < 0 ||
      !(p->max_pend > 1e-8) || !(p->start_pend > 0) || !(p->initial_tolerance > 0) || p->optimizer < 0 ||
      p->optimizer > 1 || p->calc_pp < 0 || p->calc_pp > 1 || p->prior < 0 || p->prior > 2 ||
      !(p->pp_rel_err > 0) || !(p->prior_lower >= 0) || p->pp_rule < 0 || p->pp_rule > 1 ||
      (p->pp_rule == 1 && !(p->pp_rel_err >= 50 * 2.220446049250313e-16))) {
    set_error("invalid prefs (keep_at_most 1..64, max_pend > 1e-8, tolerances > 0, optimizer 0|1, calc_pp 0|1, "
              "prior 0|1|2, pp_rel_err > 0 and with pp_rule 1 at least 50 DBL_EPSILON (GSL_EBADTOL), "
              "prior_lower >= 0, pp_rule 0|1)");
    return PGB_ERR_ARG;
  }
  return PGB_OK;
}

pgb_status pgb_queries_stage1(pgb_engine *e, const pgb_prefs *p, double *scores) {
  if (!e || !e->glvs_ready || e->Q < 1) { set_error("stage1: no GLVs or no queries"); return PGB_ERR_STATE; }
  pgb_status s;
  if ((s = check_prefs(p)) || (s = build_stage1_table(e, p->start_pend)) || (s = run_stage1(e, true))) return s;
  PGB_CUDA(cudaMemcpyAsync(scores, e->d_scores, (size_t)e->Q * e->n_edges * 8, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  return check_tc_err(e);
}

pgb_status pgb_queries_rank(pgb_engine *e, const pgb_prefs *p, int rk, int *rank) {
  if (!e || !e->glvs_ready || e->Q < 1) { set_error("rank: no GLVs or no queries"); return PGB_ERR_STATE; }
  if (rk < 1 || rk > e->n_edges || !rank) { set_error("rank: rk %d outside 1..%d", rk, e->n_edges); return PGB_ERR_ARG; }
  pgb_status s;
  if ((s = check_prefs(p))) return s;
  size_t rn = (size_t)e->Q * rk;
  if (rn > e->rank_cap) { if ((s = dalloc(&e->d_rank, rn))) return s; e->rank_cap = rn; }
  PGB_CUDA(cudaMemsetAsync(e->d_rank, 0xff, rn * sizeof(int), e->st));
  if ((s = build_stage1_table(e, p->start_pend)) || (s = run_stage1(e)) || (s = run_rank(e, rk)))
    return s;
  PGB_CUDA(cudaMemcpyAsync(rank, e->d_rank, rn * sizeof(int), cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  return check_tc_err(e);
}

pgb_status pgb_queries_run(pgb_engine *e, const pgb_prefs *p) {
  if (!e || !e->glvs_ready) { set_error("run: no GLVs"); return PGB_ERR_STATE; }
  pgb_status s;
  if ((s = check_prefs(p))) return s;
  if (e->Q < 1) return PGB_OK;
  bool all_edges = p->max_strikes == 0;
  int rk = all_edges ? e->n_edges : std::min(e->n_edges, p->max_pitches + 1 + 24);
  int maxr = all_edges ? e->n_edges : std::min(e->n_edges, p->max_pitches + 1);
  int max_sq = 1;
  for (int v : e->h_qlen) max_sq = std::max(max_sq, v);
  size_t tcap = (size_t)e->Q * std::max(8, std::min(rk, 16)) + (size_t)e->Q * p->keep_at_most + 64;
  if (all_edges) tcap = std::max(tcap, (size_t)e->Q * e->n_edges + 64);
  if (p->calc_pp) tcap += (size_t)e->Q * p->keep_at_most;  // marginal trials after the refinements
  if ((s = ensure_run_buffers(e, p, rk, maxr, tcap))) return s;
  for (int i = 0; i < 8; i++) e->counts[i] = 0;
  PGB_CUDA(cudaMemsetAsync(e->d_stats, 0, 4 * sizeof(unsigned long long), e->st));
  PGB_CUDA(cudaEventRecord(e->ev[0], e->st));
  if ((s = build_stage1_table(e, p->start_pend))) return s;
  PGB_CUDA(cudaEventRecord(e->ev[1], e->st));
  if ((s = run_stage1(e))) return s;
  PGB_CUDA(cudaEventRecord(e->ev[5], e->st));
  if ((s = run_rank(e, rk))) return s;
  PGB_CUDA(cudaEventRecord(e->ev[2], e->st));
  e->counts[0] = (double)e->Q * e->n_edges;
  // baseball rounds
  BBCtx c{};
  c.Q = e->Q; c.rk = rk; c.maxr = maxr; c.n_edges = e->n_edges; c.bins = kBins;
  c.rank = e->d_rank; c.edge_nodes = e->d_edge_nodes; c.bl = e->d_bl; c.qlen = e->d_qlen; c.qstatus = e->d_qstatus;
  c.bb = e->d_bb; c.res = e->d_res; c.tbase = e->d_tbase; c.tcount = e->d_tcount; c.trials = e->d_trials;
  c.bin_count = e->d_small + 2; c.bin_list = e->d_bin_list; c.bin_limit = e->d_small + 2 + kBins;
  c.cap_trials = (int)e->trials_cap; c.n_active = e->d_small + 1;
  c.start_pend = p->start_pend; c.tol = p->initial_tolerance; c.strike_box = p->strike_box;
  c.max_pitches = all_edges ? (1L << 40) : p->max_pitches;
  c.max_strikes = all_edges ? (1L << 40) : p->max_strikes;
  int lim[kBins];
  bin_limits(e, lim);
  int h_small[2 + 2 * kBins] = {0};
  for (int b = 0; b < kBins; b++) h_small[2 + kBins + b] = lim[b];
  if ((s = ensure_eigen_glvs(e))) return s;
  TrialCtx tc = trial_ctx(e, p, p->optimizer, 0);
  int n = e->Q;
  // Every edge of every query (max_strikes 0): the trials are independent,
  // so with fewer queries than the GPU has trial warps they run as one
  // batch of all trials rather than one query per warp
  const bool few_queries = all_edges && e->Q < 2 * kWarpTrialMinCtas * e->n_sm;
  if (whole_query_form(e) && !few_queries) return run_whole_queries(e, p, c, tc, max_sq);
  if (p->calc_pp && (s = ensure_prior_means(e, p->prior, p->prior_lower))) return s;
  k_bb_init<<<(n + 255) / 256, 256, 0, e->st>>>(c);
  PGB_LAUNCH_CHECK();
  double n_trials_total = 0;
  int rounds = 0, last_active = e->Q;
  for (int round = 0; round < 4096; round++) {
    rounds = round + 1;
    // speculative width: round 0 evaluates the minimum any query needs
    // (max_strikes + 1); later rounds are narrow since most queries that
    // continue stop within a few more pitches
    // later rounds widen as fewer queries remain: enough trials to keep every
    // SM busy for a couple of waves, at least 3 per query
    int B;
    if (all_edges) B = rk;
    else if (round == 0) B = std::min(rk, p->max_strikes + 1);
    else B = std::max(3, std::min(16, (2 * e->n_sm + last_active - 1) / std::max(1, last_active)));
    PGB_CUDA(cudaMemcpyAsync(e->d_small, h_small, sizeof(h_small), cudaMemcpyHostToDevice, e->st));
    k_bb_emit<<<(n + 255) / 256, 256, 0, e->st>>>(c, B, e->d_small);
    PGB_LAUNCH_CHECK();
    int got[2 + kBins];
    PGB_CUDA(cudaMemcpyAsync(got, e->d_small, sizeof(got), cudaMemcpyDeviceToHost, e->st));
    PGB_CUDA(cudaStreamSynchronize(e->st));
    if (got[0] == 0) break;
    n_trials_total += got[0];
    if ((s = run_bins(e, tc, got + 2, max_sq))) return s;
    k_bb_update<<<(n + 255) / 256, 256, 0, e->st>>>(c, e->d_tres);
    PGB_LAUNCH_CHECK();
    int active = 0;
    PGB_CUDA(cudaMemcpyAsync(&active, e->d_small + 1, 4, cudaMemcpyDeviceToHost, e->st));
    PGB_CUDA(cudaStreamSynchronize(e->st));
    if (active == 0) break;
    last_active = active;
  }
  PGB_CUDA(cudaEventRecord(e->ev[3], e->st));
  {  // speculation accounting: stage-2 trials emitted vs consumed by the stop rule
    std::vector<BBState> bbh(e->Q);
    PGB_CUDA(cudaMemcpyAsync(bbh.data(), e->d_bb, e->Q * sizeof(BBState), cudaMemcpyDeviceToHost, e->st));
    PGB_CUDA(cudaStreamSynchronize(e->st));
    double consumed = 0;
    for (const BBState &b : bbh) consumed += b.next;
    e->counts[4] = n_trials_total;
    e->counts[5] = consumed;
    e->counts[7] = rounds;
  }
  // keep + refine
  PGB_CUDA(cudaMemcpyAsync(e->d_small, h_small, sizeof(h_small), cudaMemcpyHostToDevice, e->st));
  k_keep_emit<<<(n + 255) / 256, 256, 0, e->st>>>(c, p->keep_at_most, log(p->keep_factor), e->d_keep_idx,
                                                  e->d_keep_n, e->d_small);
  PGB_LAUNCH_CHECK();
  int got[2 + kBins];
  PGB_CUDA(cudaMemcpyAsync(got, e->d_small, sizeof(got), cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  n_trials_total += got[0];
  e->counts[6] = got[0];
  if ((s = run_bins(e, tc, got + 2, max_sq))) return s;
  int pp_off = -1;
  if (p->calc_pp) {  // the marginal likelihood of every kept location, after all refinements
    pp_off = got[0];
    PGB_CUDA(cudaMemcpyAsync(e->d_small, h_small, sizeof(h_small), cudaMemcpyHostToDevice, e->st));
    k_pp_emit<<<(n + 255) / 256, 256, 0, e->st>>>(c, p->keep_at_most, e->d_keep_idx, e->d_keep_n, e->d_tres, pp_off,
                                                  p->prior == 1 ? 0 : 1, e->d_prior_mu);
    PGB_LAUNCH_CHECK();
    int got_pp[2 + kBins];
    PGB_CUDA(cudaMemcpyAsync(got_pp, e->d_small, sizeof(got_pp), cudaMemcpyDeviceToHost, e->st));
    PGB_CUDA(cudaStreamSynchronize(e->st));
    n_trials_total += got[0];
    if ((s = run_bins(e, tc, got_pp + 2, max_sq))) return s;
  }
  k_finalize<<<(n + 255) / 256, 256, 0, e->st>>>(c, p->keep_at_most, e->d_keep_idx, e->d_keep_n, e->d_tres, pp_off,
                                                 e->d_out, e->d_nout);
  PGB_LAUNCH_CHECK();
  PGB_CUDA(cudaEventRecord(e->ev[4], e->st));
  PGB_CUDA(cudaEventSynchronize(e->ev[4]));
  float ms;
  cudaEventElapsedTime(&ms, e->ev[1], e->ev[5]); e->t_ms[0] = ms;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]); e->t_ms[1] = ms;
  cudaEventElapsedTime(&ms, e->ev[1], e->ev[2]); e->t_ms[2] = ms;
  cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]); e->t_ms[3] = ms;
  cudaEventElapsedTime(&ms, e->ev[3], e->ev[4]); e->t_ms[4] = ms;
  cudaEventElapsedTime(&ms, e->ev[0], e->ev[4]); e->t_ms[5] = ms;
  e->counts[1] = n_trials_total;
  unsigned long long st_h[2] = {0, 0};
  PGB_CUDA(cudaMemcpy(st_h, e->d_stats, sizeof st_h, cudaMemcpyDeviceToHost));
  if ((s = check_tc_err(e))) return s;
  e->counts[2] = (double)st_h[0];
  e->counts[3] = (double)st_h[1];
  return PGB_OK;
}

// Time every (threads, window placement) shape of the trial kernel on the
// loaded queries' first-round trials, bin by bin, and keep the fastest.
pgb_status pgb_engine_autotune(pgb_engine *e, const pgb_prefs *p) {
  if (!e || !e->glvs_ready || e->Q < 1) { set_error("autotune: no GLVs or no queries"); return PGB_ERR_STATE; }
  pgb_status s;
  if ((s = check_prefs(p))) return s;
  if (warp_trials_ok(e)) {
    // the whole-query warp kernel: time its forms (matrices in registers;
    // eigenbasis at 8, 12 or 16 warps per SM) on whole runs of the loaded
    // queries, keep the fastest
    for (int b = 0; b < kBins; b++) { e->tune_threads[b] = 32; e->tune_win[b] = 0; }
    if (!warp_eig_ok(e)) { e->warp_variant = 0; return PGB_OK; }
    float best = 1e30f;
    int bv = 0;
    for (int v = 0; v < kWarpForms; v++) {
      if (v != e->warp_variant) { e->warp_variant = v; e->eig_ready = false; }
      float ms_best = 1e30f;
      for (int rep = 0; rep < 2; rep++) {
        if ((s = pgb_queries_run(e, p))) return s;
        ms_best = std::min(ms_best, (float)e->t_ms[3]);
      }
      if (ms_best < best) { best = ms_best; bv = v; }
    }
    if (bv != e->warp_variant) { e->warp_variant = bv; e->eig_ready = false; }
    return PGB_OK;
  }
  bool all_edges = p->max_strikes == 0;
  int rk = all_edges ? e->n_edges : std::min(e->n_edges, p->max_pitches + 1 + 24);
  int maxr = all_edges ? e->n_edges : std::min(e->n_edges, p->max_pitches + 1);
  int max_sq = 1;
  for (int v : e->h_qlen) max_sq = std::max(max_sq, v);
  size_t tcap = (size_t)e->Q * std::max(8, std::min(rk, 16)) + (size_t)e->Q * p->keep_at_most + 64;
  if (all_edges) tcap = std::max(tcap, (size_t)e->Q * e->n_edges + 64);
  if ((s = ensure_run_buffers(e, p, rk, maxr, tcap)) || (s = build_stage1_table(e, p->start_pend)) ||
      (s = run_stage1(e)) || (s = run_rank(e, rk)))
    return s;
  BBCtx c{};
  c.Q = e->Q; c.rk = rk; c.maxr = maxr; c.n_edges = e->n_edges; c.bins = kBins;
  c.rank = e->d_rank; c.edge_nodes = e->d_edge_nodes; c.bl = e->d_bl; c.qlen = e->d_qlen; c.qstatus = e->d_qstatus;
  c.bb = e->d_bb; c.res = e->d_res; c.tbase = e->d_tbase; c.tcount = e->d_tcount; c.trials = e->d_trials;
  c.bin_count = e->d_small + 2; c.bin_list = e->d_bin_list; c.bin_limit = e->d_small + 2 + kBins;
  c.cap_trials = (int)e->trials_cap; c.n_active = e->d_small + 1;
  c.start_pend = p->start_pend; c.tol = p->initial_tolerance; c.strike_box = p->strike_box;
  c.max_pitches = all_edges ? (1L << 40) : p->max_pitches;
  c.max_strikes = all_edges ? (1L << 40) : p->max_strikes;
  int lim[kBins];
  bin_limits(e, lim);
  int h_small[2 + 2 * kBins] = {0};
  for (int b = 0; b < kBins; b++) h_small[2 + kBins + b] = lim[b];
  k_bb_init<<<(e->Q + 255) / 256, 256, 0, e->st>>>(c);
  PGB_LAUNCH_CHECK();
  PGB_CUDA(cudaMemcpyAsync(e->d_small, h_small, sizeof(h_small), cudaMemcpyHostToDevice, e->st));
  int B = all_edges ? rk : std::min(rk, p->max_strikes + 1);
  k_bb_emit<<<(e->Q + 255) / 256, 256, 0, e->st>>>(c, B, e->d_small);
  PGB_LAUNCH_CHECK();
  int got[2 + kBins];
  PGB_CUDA(cudaMemcpyAsync(got, e->d_small, sizeof(got), cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  if ((s = ensure_eigen_glvs(e))) return s;
  TrialCtx tc = trial_ctx(e, p, p->optimizer, 0);
  tc.stats = nullptr;
  const int cand_threads[4] = {32, kTuneTc, 256, 128};
  for (int b = 0; b < kBins; b++) {
    int n = got[2 + b];
    if (n == 0) continue;
    float best = 1e30f;
    int bt = e->tune_threads[b], bw = e->tune_win[b];
    for (int ti = 0; ti < 4; ti++)
      for (int w = 1; w >= 0; w--) {
        int cap;
        bool win;
        if (cand_threads[ti] == 32 && !warp_form_ok(e)) continue;
        if (cand_threads[ti] == kTuneTc && !tc_trials_ok(e)) continue;
        // the warp and tensor-core kernels read the windows from L2
        if ((cand_threads[ti] == 32 || cand_threads[ti] == kTuneTc) && w == 1) continue;
        bin_shape(e, b, max_sq, w, &cap, &win);
        if (w == 1 && !win) continue;  // window does not fit: same as w == 0
        float ms_best = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
          PGB_CUDA(cudaEventRecord(e->ev[6], e->st));
          if ((s = launch_trials(e, e->st, tc, e->d_bin_list + (long)b * e->trials_cap, n, cap, win, e->d_tres,
                                 cand_threads[ti])))
            return s;
          PGB_CUDA(cudaEventRecord(e->ev[7], e->st));
          PGB_CUDA(cudaEventSynchronize(e->ev[7]));
          float ms;
          cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]);
          ms_best = std::min(ms_best, ms);
        }
        if (ms_best < best) { best = ms_best; bt = cand_threads[ti]; bw = w; }
      }
    e->tune_threads[b] = bt;
    e->tune_win[b] = bw;
  }
  // In a run the bins execute concurrently, so a form that loses on a bin
  // alone can win on the whole round (its tail overlaps the other bins).
  // Time the whole round for the per-bin choice and for each uniform form.
  // Only forms with one CTA size in every bin are kept: those run as whole
  // queries (no speculative rounds), which the round timing understates.
  int per_bin_t[kBins], per_bin_w[kBins];
  bool per_bin_uniform = true;
  for (int b = 0; b < kBins; b++) {
    per_bin_t[b] = e->tune_threads[b];
    per_bin_w[b] = e->tune_win[b];
    if (per_bin_t[b] != per_bin_t[0]) per_bin_uniform = false;
  }
  const int uni_t[4] = {32, kTuneTc, 128, 256}, uni_w[4] = {0, 0, 1, 1};
  float best = 1e30f;
  int best_cfg = -2;
  for (int cfg = -1; cfg < 4; cfg++) {
    if (cfg == -1 && !per_bin_uniform) continue;
    if (cfg == 0 && !warp_form_ok(e)) continue;
    if (cfg == 1 && !tc_trials_ok(e)) continue;
    for (int b = 0; b < kBins; b++) {
      e->tune_threads[b] = cfg < 0 ? per_bin_t[b] : uni_t[cfg];
      e->tune_win[b] = cfg < 0 ? per_bin_w[b] : uni_w[cfg];
    }
    float ms_best = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      PGB_CUDA(cudaEventRecord(e->ev[6], e->st));
      if ((s = run_bins(e, tc, got + 2, max_sq))) return s;
      PGB_CUDA(cudaEventRecord(e->ev[7], e->st));
      PGB_CUDA(cudaEventSynchronize(e->ev[7]));
      float ms;
      cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]);
      ms_best = std::min(ms_best, ms);
    }
    if (ms_best < best) { best = ms_best; best_cfg = cfg; }
  }
  for (int b = 0; b < kBins; b++) {
    e->tune_threads[b] = best_cfg < 0 ? per_bin_t[b] : uni_t[best_cfg];
    e->tune_win[b] = best_cfg < 0 ? per_bin_w[b] : uni_w[best_cfg];
  }
  if (best_cfg == 0 && warp_cat_ok(e) && e->eig_ok) {
    // the CAT warp form: its matrix, eigenbasis and packed eigenbasis
    // variants on whole runs
    float bf = 1e30f;
    int bv = 0;
    for (int v = 0; v < kCatForms; v++) {
      if (v != e->warp_variant) { e->warp_variant = v; e->eig_ready = false; }
      float ms_best = 1e30f;
      for (int rep = 0; rep < 2; rep++) {
        if ((s = pgb_queries_run(e, p))) return s;
        ms_best = std::min(ms_best, (float)e->t_ms[3]);
      }
      if (ms_best < bf) { bf = ms_best; bv = v; }
    }
    if (bv != e->warp_variant) { e->warp_variant = bv; e->eig_ready = false; }
  }
  return check_tc_err(e);
}

pgb_status pgb_engine_get_tuning(pgb_engine *e, int *threads, int *smem_windows) {
  if (!e) return PGB_ERR_ARG;
  for (int b = 0; b < kBins; b++) {
    threads[b] = e->tune_threads[b];
    smem_windows[b] = e->tune_threads[b] == 32 && (warp_trials_ok(e) || warp_cat_ok(e))
                          ? e->warp_variant
                          : e->tune_win[b];
  }
  return PGB_OK;
}

pgb_status pgb_engine_set_tuning(pgb_engine *e, const int *threads, const int *smem_windows) {
  if (!e || !threads || !smem_windows) { set_error("set_tuning: null argument"); return PGB_ERR_ARG; }
  const bool warp_forms = warp_trials_ok(e);
  for (int b = 0; b < kBins; b++) {
    const bool wf = threads[b] == 32 && warp_forms;  // smem_windows selects the warp form
    const bool cf = threads[b] == 32 && warp_cat_ok(e);  // ... or the CAT warp form
    if ((threads[b] != 32 && threads[b] != kTuneTc && threads[b] != 128 && threads[b] != 256) ||
        (!wf && !cf && (smem_windows[b] & ~1)) || (wf && (smem_windows[b] < 0 || smem_windows[b] >= kWarpForms)) ||
        (cf && (smem_windows[b] < 0 || smem_windows[b] >= kCatForms)) ||
        (wf && smem_windows[b] > 0 && !warp_eig_ok(e))) {
      set_error("set_tuning: bin %d: threads must be 1, 32, 128 or 256 and smem_windows 0 or 1 (for the "
                "nucleotide Gamma warp form 0 .. 5 where the eigenbasis forms apply, for the CAT warp "
                "form 0 .. 2)", b);
      return PGB_ERR_ARG;
    }
  }
  if (threads[0] == 32 && warp_cat_ok(e) && smem_windows[0] != 0 && !e->eig_ok) {
    set_error("set_tuning: the CAT eigenbasis form needs a rate matrix with one zero eigenvalue");
    return PGB_ERR_ARG;
  }
  for (int b = 0; b < kBins; b++) {
    e->tune_threads[b] = threads[b];
    e->tune_win[b] = threads[b] == 32 && (warp_forms || warp_cat_ok(e)) ? 0 : smem_windows[b];
  }
  // smem_windows of a warp bin selects the form: the nucleotide Gamma forms
  // 0 .. 5, or the CAT form (0 matrices per category, 1 the eigenbasis, 2
  // the eigenbasis on packed FP32 pairs)
  const bool cat_forms = warp_cat_ok(e);
  if (threads[0] == 32 && (warp_forms || cat_forms) && smem_windows[0] != e->warp_variant) {
    e->warp_variant = smem_windows[0];
    e->eig_ready = false;  // the eigen-coordinate layout follows the form
  }
  return PGB_OK;
}

pgb_status pgb_queries_fetch(pgb_engine *e, pgb_placement *out, int *n_out, int *qstatus) {
  if (!e || e->Q < 1) return PGB_OK;
  if (!e->d_out) { set_error("fetch: nothing run"); return PGB_ERR_STATE; }
  PGB_CUDA(cudaMemcpyAsync(out, e->d_out, (size_t)e->Q * e->out_keep * sizeof(pgb_placement), cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaMemcpyAsync(n_out, e->d_nout, (size_t)e->Q * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaMemcpyAsync(qstatus, e->d_qstatus, (size_t)e->Q * 4, cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  return PGB_OK;
}

pgb_status pgb_place_batch(pgb_engine *e, const pgb_prefs *p, int n_queries, const char *seqs, int batch,
                           pgb_placement *out, int *n_out, int *qstatus) {
  if (!e || !p || n_queries < 0 || batch < 0 || (n_queries > 0 && (!seqs || !out || !n_out || !qstatus))) {
    set_error("place: bad argument");
    return PGB_ERR_ARG;
  }
  if (batch == 0) {
    // Automatic device batches: per query the stage-1 pairs (8 bytes per
    // edge, and 8 more for the FP64 rows of queries with ambiguity
    // characters) and ~12 bytes per site of query buffers (characters,
    // codes, the masked-site lists, the stage-1 site classes) stay within
    // 8 GiB, a small part of the GPU's memory; fewer batches mean fewer
    // stage-1 launches and fewer whole-query tails.
    const long per_q = 16L * e->n_edges + 12L * e->S + 256;
    batch = (int)std::max(1024L, std::min(65536L, (8L << 30) / per_q));
    if (const char *env = getenv("PGB_PLACE_BATCH")) batch = std::max(1, atoi(env));  // override (tests, tuning)
  }
  pgb_status s;
  if (n_queries == 0) return pgb_queries_load(e, 0, seqs);
  for (int b0 = 0; b0 < n_queries; b0 += batch) {
    const int nb = std::min(batch, n_queries - b0);
    if ((s = pgb_queries_load(e, nb, seqs + (size_t)b0 * e->S)) || (s = pgb_queries_run(e, p)) ||
        (s = pgb_queries_fetch(e, out + (size_t)b0 * p->keep_at_most, n_out + b0, qstatus + b0)))
      return s;
  }
  return PGB_OK;
}

pgb_status pgb_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) { set_error("host_alloc: null pointer"); return PGB_ERR_ARG; }
  *ptr = nullptr;
  PGB_CUDA(cudaHostAlloc(ptr, std::max<size_t>(bytes, 1), cudaHostAllocPortable));
  return PGB_OK;
}

pgb_status pgb_host_free(void *ptr) {
  if (ptr) PGB_CUDA(cudaFreeHost(ptr));
  return PGB_OK;
}

pgb_status pgb_place(pgb_engine *e, const pgb_prefs *p, int n_queries, const char *seqs, pgb_placement *out,
                     int *n_out, int *qstatus) {
  return pgb_place_batch(e, p, n_queries, seqs, 0, out, n_out, qstatus);
}

pgb_status pgb_queries_trials(pgb_engine *e, const pgb_prefs *p, int optimizer, int mode, int n_trials,
                              const pgb_trial *trials, pgb_trial_out *out) {
  if (!e || !e->glvs_ready || e->Q < 1) { set_error("trials: no GLVs or no queries"); return PGB_ERR_STATE; }
  pgb_status s;
  if ((s = check_prefs(p))) return s;
  if (optimizer < 0 || optimizer > 1 || mode < 0 || mode > 2 || n_trials < 0) { set_error("trials: bad mode"); return PGB_ERR_ARG; }
  if (!n_trials) return PGB_OK;
  if (mode == 2 && (s = ensure_prior_means(e, p->prior, p->prior_lower))) return s;
  std::vector<TrialIn> tin(n_trials);
  int max_sq = 1;
  for (int i = 0; i < n_trials; i++) {
    const pgb_trial &t = trials[i];
    if (t.query < 0 || t.query >= e->Q || t.edge < 0 || t.edge >= e->n_nodes || t.edge == e->root) {
      set_error("trials: trial %d out of range", i);
      return PGB_ERR_ARG;
    }
    if (e->h_qlen[t.query] < 1) { set_error("trials: query %d has no informative site", t.query); return PGB_ERR_ARG; }
    tin[i] = TrialIn{t.query, t.edge, t.pend0, t.dist0, t.tol};
    if (mode == 2) {
      tin[i].prior_kind = p->prior == 1 ? 0 : 1;
      tin[i].prior_mu = e->h_prior_mu[t.edge];
    }
    max_sq = std::max(max_sq, e->h_qlen[t.query]);
  }
  if ((size_t)n_trials > e->trials_cap) {
    if ((s = dalloc(&e->d_trials, n_trials)) || (s = dalloc(&e->d_tres, n_trials)) ||
        (s = dalloc(&e->d_bin_list, (size_t)n_trials * kBins)))
      return s;
    e->trials_cap = n_trials;
  }
  PGB_CUDA(cudaMemcpyAsync(e->d_trials, tin.data(), n_trials * sizeof(TrialIn), cudaMemcpyHostToDevice, e->st));
  // bin on the host
  int lim[kBins];
  bin_limits(e, lim);
  std::vector<std::vector<int>> bins(kBins);
  for (int i = 0; i < n_trials; i++) {
    int sq = e->h_qlen[tin[i].q], b = 0;
    while (b < kBins - 1 && sq > lim[b]) b++;
    bins[b].push_back(i);
  }
  int counts[kBins];
  for (int b = 0; b < kBins; b++) {
    counts[b] = (int)bins[b].size();
    if (counts[b])
      PGB_CUDA(cudaMemcpyAsync(e->d_bin_list + (size_t)b * e->trials_cap, bins[b].data(), counts[b] * 4,
                               cudaMemcpyHostToDevice, e->st));
  }
  if ((s = ensure_eigen_glvs(e))) return s;
  TrialCtx tc = trial_ctx(e, p, optimizer, mode);
  if ((s = run_bins(e, tc, counts, max_sq))) return s;
  std::vector<TrialRes> res(n_trials);
  PGB_CUDA(cudaMemcpyAsync(res.data(), e->d_tres, n_trials * sizeof(TrialRes), cudaMemcpyDeviceToHost, e->st));
  PGB_CUDA(cudaStreamSynchronize(e->st));
  if ((s = check_tc_err(e))) return s;
  for (int i = 0; i < n_trials; i++) {
    out[i].like = res[i].like;
    out[i].pend = res[i].pend;
    out[i].dist = res[i].dist;
    for (int k = 0; k < 6; k++) out[i].derivs[k] = res[i].der[k];
    out[i].status = res[i].status;
    out[i].n_evals = res[i].n_evals;
  }
  return PGB_OK;
}

pgb_status pgb_engine_timings(pgb_engine *e, double *ms, double *counts) {
  if (!e) return PGB_ERR_ARG;
  for (int i = 0; i < 6; i++) ms[i] = e->t_ms[i];
  for (int i = 0; i < 8; i++) counts[i] = e->counts[i];
  return PGB_OK;
}

}  // extern "C"
