/*
 * pplacer_gb300 -- C ABI of the GB300 (sm_103a) placement-likelihood engine.
 *
 * Two layers, both plain C: pointers, sizes and status codes only.
 *
 * 1. The plain drop-in (pgb_* functions named after the linear_c.c symbol they
 *    replace).  Each one has the argument meaning and order of the OCaml
 *    external in pplacer_src/linear.ml:13-89; the OCaml bigarray dimensions
 *    (Caml_ba_array_val(v)->dim[i]) become explicit int arguments.  All
 *    pointers are HOST pointers to C-contiguous float64 / uint16 arrays with
 *    the layout stated at pplacer_src/linear_c.c:6-12 (matrices [site][state],
 *    tensors [rate][site][state]).  Each call copies its inputs to the GPU,
 *    runs one sm_103a kernel in FP64 and copies the result back, so the
 *    OCaml side keeps the FP64 values and exponent handling it relies on.
 *    Like the reference, dimension mismatches are the caller's business and
 *    log(0) yields -inf silently.  The CUDA context is created lazily on the
 *    first call, so a process may fork before its first call (pplacer's
 *    worker processes, pplacer_src/multiprocessing.ml:120-152).
 *
 * 2. The batched engine (pgb_engine_*): device-resident reference GLVs and
 *    whole-query placement (pplacer_src/core.ml:113-409) in FP32 with exact
 *    int32 per-site scaling exponents, stage-1 ranking, the baseball
 *    heuristic, Brent or safeguarded-Newton branch-length optimisation and
 *    the final refinement, for the Gamma-mixture (pplacer_src/gmix_model.ml)
 *    and per-site CAT (pplacer_src/gcat_model.ml) models.
 *
 * Every function returns a pgb_status (or, for the drop-in log functions, the
 * double result); pgb_last_error() describes the last failure of the calling
 * thread.  A missing or unusable GPU is an error, never a silent CPU path.
 */
#ifndef PPLACER_GB300_H
#define PPLACER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PGB_OK = 0,
  PGB_ERR_ARG = 1,       /* invalid argument or size */
  PGB_ERR_CUDA = 2,      /* CUDA runtime failure (no GPU, launch error, ...) */
  PGB_ERR_NOMEM = 3,     /* device or host allocation failed */
  PGB_ERR_STATE = 4,     /* call out of order (e.g. place before GLVs exist) */
  PGB_ERR_QUERY = 5      /* query-level failure; see the per-query status */
} pgb_status;

const char *pgb_last_error(void);
/* Number of kernels this library launched on the calling process's streams. */
uint64_t pgb_kernel_launch_count(void);

/* ----------------------------------------------------------------------------
 * 1. Plain drop-in for pplacer_src/linear_c.c
 * ------------------------------------------------------------------------- */

/* gemmish_c (linear_c.c:29-90; linear.ml:13): dst[s,i] = sum_j a[i,j] b[s,j] */
pgb_status pgb_gemmish(double *dst, const double *a, const double *b, int n_sites, int n_states);

/* dediagonalize (linear_c.c:92-146; linear.ml:19):
 * dst[i,j] = sum_k lambda[k] u[i,k] uit[j,k] */
pgb_status pgb_dediagonalize(double *dst, const double *u, const double *lambda, const double *uit, int n);

/* mat_log_like3_c (linear_c.c:170-216; linear.ml:28) */
double pgb_mat_log_like3(const double *statd, const double *x, const double *y, const double *z, int n_sites,
                         int n_states);

/* mat_pairwise_prod_c (linear_c.c:218-230; linear.ml:31) */
pgb_status pgb_mat_pairwise_prod(double *dst, const double *x, const double *y, int n_sites, int n_states);

/* mat_statd_pairwise_prod_c (linear_c.c:232-249; linear.ml:34) */
pgb_status pgb_mat_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                       int n_sites, int n_states);

/* mat_masked_logdot_c (linear_c.c:251-296; linear.ml:40) */
double pgb_mat_masked_logdot(const double *x, const double *y, const uint16_t *mask, int n_sites, int n_states);

/* mat_bounded_logdot_c (linear_c.c:298-340; linear.ml:46) */
double pgb_mat_bounded_logdot(const double *x, const double *y, int first, int last, int n_sites, int n_states);

/* ten_log_like3_c (linear_c.c:367-424; linear.ml:55); util: n_sites scratch
 * that receives the per-site likelihoods summed over rates, as the reference. */
double pgb_ten_log_like3(const double *statd, const double *x, const double *y, const double *z, double *util,
                         int n_rates, int n_sites, int n_states);

/* ten_pairwise_prod_c (linear_c.c:426-441; linear.ml:58) */
pgb_status pgb_ten_pairwise_prod(double *dst, const double *x, const double *y, int n_rates, int n_sites,
                                 int n_states);

/* ten_statd_pairwise_prod_c (linear_c.c:443-463; linear.ml:61) */
pgb_status pgb_ten_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                       int n_rates, int n_sites, int n_states);

/* ten_masked_logdot_c (linear_c.c:465-539; linear.ml:67) */
double pgb_ten_masked_logdot(const double *x, const double *y, const uint16_t *mask, double *util, int n_rates,
                             int n_sites, int n_states);

/* ten_bounded_logdot_c (linear_c.c:541-605; linear.ml:73) */
double pgb_ten_bounded_logdot(const double *x, const double *y, int first, int last, double *util, int n_rates,
                              int n_sites, int n_states);

/* vec_pairwise_prod_c (linear_c.c:607-618; linear.ml:76) */
pgb_status pgb_vec_pairwise_prod(double *dst, const double *x, const double *y, int n);

/* int_vec_tot_c (linear_c.c:620-630; linear.ml:80) */
int pgb_int_vec_tot(const uint16_t *x, int n);

/* int_vec_pairwise_prod_c (linear_c.c:632-642; linear.ml:83): uint16 wraps */
pgb_status pgb_int_vec_pairwise_prod(uint16_t *dst, const uint16_t *x, const uint16_t *y, int n);

/* float_mat_int_vec_mul_c (linear_c.c:644-670; linear.ml:89):
 * dst[j] += sum_i mat[i,j] vec[i], mat is n x k.  The reference's
 * caml_failwith on mismatched sizes is the stub's job (it has the dims). */
pgb_status pgb_float_mat_int_vec_mul(double *dst, const double *mat, const uint16_t *vec, int n, int k);

/* Allocation-free ten_log_like3 on device buffers.  No counterpart in the
 * reference: it is for callers that cannot allocate device memory when they
 * need a likelihood -- their GPU memory belongs to another runtime's pool, or
 * they allocate only at start-up.  statd ([n_states]), x, y, z
 * ([n_rates][n_sites][n_states]) and result (one double) are DEVICE pointers;
 * stream is a cudaStream_t (NULL: the default stream) and the call is
 * asynchronous on it.  The reduction's scratch is a fixed array inside the
 * library, held by every GPU that loads it: n_sites <= 65,536, larger sizes
 * return PGB_ERR_ARG.  All calls on a device share that array, so calls that
 * overlap on the GPU race.  The first call on a device, and the first call
 * after that device's context was reset (cudaDeviceReset), looks up the
 * array's address; make it before any stream capture.  Calls no cudaMalloc or
 * cudaFree. */
pgb_status pgb_ten_log_like3_noalloc(const double *statd, const double *x, const double *y, const double *z,
                                     int n_rates, int n_sites, int n_states, double *result, void *stream);

/* FP32 evolve on the tensor cores: out[s][i] = sum_j b[i][j] a[s][j] for
 * s < n_rows, i < n_out (<= 64), j < n_states (<= 24) -- the per-site
 * matrix-vector product of gemmish_c (linear_c.c:29-90) with the sites as
 * rows, computed as the 20-state trial kernel computes it (tcgen05 MMAs of
 * 128 sites, operands split into TF32 hi + lo, three products accumulated in
 * FP32).  Host pointers, row-major; synchronous.  No counterpart in the
 * reference (which evolves in FP64 on the CPU): it exposes the trial kernel's
 * arithmetic for checks. */
pgb_status pgb_tc_evolve(const float *a, const float *b, float *out, int n_rows, int n_states, int n_out);

/* ----------------------------------------------------------------------------
 * 2. Batched placement engine
 * ------------------------------------------------------------------------- */

typedef struct pgb_engine pgb_engine;

/* Model (the fields of Gmix_model.Model.t / Gcat_model.Model.t,
 * gmix_model.ml:10-16, gcat_model.ml:33-41): Diagd x, lambda, xit
 * (diagd.ml:33-39) with x diag(lambda) x^-1 the rate matrix; statd; the
 * Gamma category rates (Gmix) or the CAT category rates (Gcat). */
typedef struct {
  int n_states;               /* 4 (nucleotide) or 20 (amino acid) */
  int n_rates;                /* Gamma categories, or CAT categories */
  int gcat;                   /* 0: Gamma mixture; 1: per-site CAT categories */
  int n_sites;                /* pre-masked alignment length */
  const double *statd;        /* [n_states] */
  const double *x;            /* [n_states * n_states] */
  const double *lambda;       /* [n_states] */
  const double *xit;          /* [n_states * n_states] */
  const double *rates;        /* [n_rates] */
  const int *site_categories; /* [n_sites] CAT category of each site (gcat), else NULL */
} pgb_model_desc;

/* Reference tree: n_nodes nodes numbered post-order (children before parents,
 * children of a node in increasing id order -- pplacer's Newick numbering,
 * newick_parser.mly:50-59); parent[root] = -1; bl[i] = length of the edge
 * above node i (the root's is taken as 0, newick_gtree.ml:145-157). */
typedef struct {
  int n_nodes;
  const int *parent;
  const double *bl;
} pgb_tree_desc;

pgb_status pgb_engine_create(const pgb_model_desc *model, const pgb_tree_desc *tree, pgb_engine **out);
pgb_status pgb_engine_destroy(pgb_engine *e);

/* Compute darr / parr / snodes on the GPU from the reference alignment
 * (Like_stree.calc_distal_and_proximal, like_stree.ml:43-110; pull exponents
 * at -10 and Glv_arr.prep_supernodes, pplacer_run.ml:332-340).  leaf_row[i] is
 * the row of leaf i in seqs (n_rows x n_sites characters), -1 for inner nodes.
 * Arithmetic in FP64; the placement copies are then stored in FP32 with int32
 * exponents. */
pgb_status pgb_engine_precompute(pgb_engine *e, const int *leaf_row, const char *seqs, int n_rows);

/* Site-category refinement of a per-site category model (Gcat_model.refine,
 * gcat_model.ml:387-419; run by pplacer_run.ml:316-317 when the alignment
 * comes from the input): for every category, the per-site log likelihood of
 * the whole tree with every site in it, scored ll + 2 log(rate) - 3 rate;
 * each site takes the first best category.  The engine's categories are
 * replaced (written to categories[n_sites] when not NULL), and its GLVs must
 * be computed again (pgb_engine_precompute) before placing.  Arguments as
 * pgb_engine_precompute. */
pgb_status pgb_engine_refine_categories(pgb_engine *e, const int *leaf_row, const char *seqs, int n_rows,
                                        int *categories);

/* Upload darr / parr / snodes that the caller computed (FP64 GLVs
 * [n_nodes][R][n_sites][n_states] with int32 exponents [n_nodes][n_sites]; R
 * is 1 for gcat).  snodes may be NULL, in which case they are rebuilt on the
 * GPU from darr and parr. */
pgb_status pgb_engine_set_glvs(pgb_engine *e, const double *darr, const int *darr_e, const double *parr,
                               const int *parr_e, const double *snodes, const int *snodes_e);

/* Read back one GLV of the stored FP32 copies as FP64 (which: 0 darr, 1 parr,
 * 2 snode); a: [R][n_sites][n_states], ex: [n_sites]. */
pgb_status pgb_engine_get_glv(pgb_engine *e, int which, int node, double *a, int *ex);

/* Placement preferences (pplacer_src/prefs.ml:76-114 defaults in brackets). */
typedef struct {
  double start_pend;         /* [0.1] */
  double max_pend;           /* [2.0] */
  double initial_tolerance;  /* [0.01] stage-2 tolerance; the final pass uses 1e-5 (core.ml:14) */
  int max_strikes;           /* [6]; 0 evaluates every edge */
  double strike_box;         /* [3.0] */
  int max_pitches;           /* [40] */
  int keep_at_most;          /* [7] */
  double keep_factor;        /* [0.01] */
  int optimizer;             /* 0: Brent as the reference (minimization.ml:83-101);
                                1: batched safeguarded Newton on the adjoint */
  int calc_pp;               /* [0] posterior probabilities (-p, core.ml:378-401): one
                                marginal-likelihood trial per kept location after its
                                refinement; every model and trial kernel */
  int prior;                 /* [0] pendant prior: 0 exponential with mean = tree length / edges,
                                1 uniform (--unif-prior), 2 informative exponential
                                (--inform-prior, core.ml:34-51) */
  double pp_rel_err;         /* [0.01] relative error of the QNG integrals (pp_rule 1) */
  double prior_lower;        /* [0.0] added to the informative prior's means (--prior-lower) */
  int pp_rule;               /* [0] the marginal likelihood's quadrature: 0 Gauss-Legendre
                                panels around the optimum (accurate to ~1e-3 in log units);
                                1 the reference's own computation, Three_tax.calc_marg_prob
                                (three_tax.ml:124-215): find_upper_limit's Brent search,
                                nested QNG (Gsl.Integration.qng) to pp_rel_err, and on
                                ETOL the upper limit halved and the integral retried, at
                                most 10 times */
} pgb_prefs;

void pgb_prefs_default(pgb_prefs *p);

/* One placement (pplacer_src/placement.ml:168-175 fields). */
typedef struct {
  int edge;       /* edge_num: node id below the edge */
  int pad;
  double like;    /* likelihood (log) */
  double lwr;     /* like_weight_ratio */
  double dist;    /* distal_length */
  double pend;    /* pendant_length */
  double marginal_like;  /* marginal_like (calc_pp), else NaN */
  double post_prob;      /* post_prob (calc_pp), else NaN */
} pgb_placement;

/* Per-query status codes. */
enum {
  PGB_Q_OK = 0,
  PGB_Q_NO_INFORMATIVE = 1, /* no informative site (core.ml:157-158) */
  PGB_Q_EMPTY = 2,          /* every location failed (core.ml:319-321) */
  PGB_Q_BAD_CHAR = 3,       /* unknown character (pplacer_run.ml:63-69) */
  PGB_Q_START_FAILURE = 4   /* Brent start finder failure (minimization.ml:11-13,35-36) */
};

/* Place n_queries pre-masked query rows (n_queries x n_sites characters, host
 * memory).  out: n_queries * keep_at_most slots, sorted by like_weight_ratio
 * as Pquery.make_ml_sorted (pquery.ml:86-92); n_out[q] placements written;
 * qstatus[q] a PGB_Q_* code.  Host buffers in, host buffers out.  Large
 * query sets run in device batches (1,024 to 65,536 queries, sized so the
 * stage-1 buffers of a batch stay within 8 GiB; the environment variable
 * PGB_PLACE_BATCH overrides the size).  Replaces the per-query placement of
 * Core.pplacer_core (core.ml:113-409) and the forked workers. */
pgb_status pgb_place(pgb_engine *e, const pgb_prefs *prefs, int n_queries, const char *seqs, pgb_placement *out,
                     int *n_out, int *qstatus);

/* pgb_place with the caller's device batch size: batch queries are loaded,
 * placed and fetched at a time (0: the automatic size of pgb_place). */
pgb_status pgb_place_batch(pgb_engine *e, const pgb_prefs *prefs, int n_queries, const char *seqs, int batch,
                           pgb_placement *out, int *n_out, int *qstatus);

/* Page-locked host memory for the query and result buffers of pgb_place /
 * pgb_place_batch: copies from and to it run at the host link's full rate
 * instead of through the driver's staging buffers.  pgb_host_free releases
 * a buffer of pgb_host_alloc.  No counterpart in the reference (its buffers
 * are OCaml bigarrays, gstar_support.ml:100-115); a caller that keeps its
 * query rows in such a buffer passes it to pgb_place_batch unchanged. */
pgb_status pgb_host_alloc(size_t bytes, void **ptr);
pgb_status pgb_host_free(void *ptr);

/* The same placement split so the device part can be timed alone: load
 * queries to the device, run the placement on them (no host traffic), fetch
 * the results. */
pgb_status pgb_queries_load(pgb_engine *e, int n_queries, const char *seqs);
pgb_status pgb_queries_run(pgb_engine *e, const pgb_prefs *prefs);
pgb_status pgb_queries_fetch(pgb_engine *e, pgb_placement *out, int *n_out, int *qstatus);

/* Stage 1 alone on the loaded queries (Glv.masked_logdot against every
 * supernode, core.ml:187-197): scores[q][i] for the i-th non-root node in
 * increasing id order. */
pgb_status pgb_queries_stage1(pgb_engine *e, const pgb_prefs *prefs, double *scores);

/* Stage 1 and its ranking (core.ml:195-197, fig.ml:143-147): rank[q][r] for
 * r < rk (rk <= the number of edges) is the index, in the order of
 * pgb_queries_stage1's columns, of the query's r-th best edge: scores
 * descending, equal scores by increasing index, NaN below every number. */
pgb_status pgb_queries_rank(pgb_engine *e, const pgb_prefs *prefs, int rk, int *rank);

/* Branch-length optimisation of explicit (query, location) trials on the
 * loaded queries (Three_tax.optimize from the given start, core.ml:255-279 with
 * the retry from default lengths).  optimizer: 0 Brent, 1 Newton;
 * mode 0 optimises, mode 1 only evaluates logL and its derivatives at the
 * start point (the forward/backward pair), mode 2 computes the marginal
 * likelihood around the start point, which must be the location's optimum
 * (Three_tax.calc_marg_prob, three_tax.ml:169-215; prefs.prior selects the
 * pendant prior; the result is in like).  Outputs per trial:
 * like, pend, dist, status (0 ok, 1 max-iter, 2 failed), n_evals, and
 * derivs[6] = dL/dpend, dL/ddist, d2L/dpend2, d2L/ddist2, d2L/dpend ddist,
 * (unused) at the final point. */
typedef struct {
  int query;
  int edge;
  double pend0, dist0;
  double tol;
} pgb_trial;

typedef struct {
  double like, pend, dist;
  double derivs[6];
  int status;
  int n_evals;
} pgb_trial_out;

pgb_status pgb_queries_trials(pgb_engine *e, const pgb_prefs *prefs, int optimizer, int mode, int n_trials,
                              const pgb_trial *trials, pgb_trial_out *out);

/* Autotuner of the stage-2 trial kernel, timed on whole placement runs of
 * the loaded queries.  Nucleotide models whose Gamma mixture has 1, 2, 4 or
 * 8 rates use the whole-query warp kernel (one warp runs a query's baseball
 * trials, keep and refinement) in one of six forms, which autotune times and
 * picks from: 0 the transition matrices in registers (8 warps per SM); 1, 2,
 * 3 the eigenbasis form (eigen-coordinate windows) at 8, 12 and 16 warps per
 * SM; 4, 5 the eigenbasis form on packed FP32 pairs at 12 and 16 (the
 * default is 4).  For the other models (CAT and 20 states): for each of the
 * 6 query-length bins (<= 256, 512, 768, 1024, 1536 informative sites,
 * longer; 128, 256, 384, 512, 640 for 20 states and CAT), time the warp form
 * (CAT), one CTA of 128 or 256 threads per trial with the query's sites of
 * darr / parr staged in shared memory or read from L2, and for 20-state
 * Gamma mixtures the tensor-core team (tcgen05 evolves), on the loaded
 * queries' first baseball round; then time the whole round for that choice
 * and for each uniform form, keep the fastest one with a single CTA size in
 * every bin, and for a CAT warp choice time its three forms (0 matrices per
 * category, 1 the eigenbasis, 2 the eigenbasis on packed FP32 pairs, the
 * default).  get_tuning reports the table (threads[6], smem_windows[6]: for a
 * warp bin the form); set_tuning imposes one (threads 1 = tensor-core team,
 * 32, 128 or 256; smem_windows 0 or 1, 0 .. 5 for the nucleotide Gamma warp
 * forms, 0 .. 2 for the CAT warp forms).  When every bin has the
 * same threads, pgb_queries_run places whole queries in one persistent
 * launch (a warp, a tensor-core team or a CTA per query, windows as bin 0
 * says) -- except every-edge runs (max_strikes 0) of fewer queries than the
 * GPU has trial warps, which run all their trials as one batch; otherwise it
 * runs the baseball in speculative rounds of per-trial CTAs.  Where the warp
 * or tensor-core form does not apply it falls back to 256.  20-state Gamma
 * mixtures start with the tensor-core form.  No reference counterpart:
 * pplacer has one CPU code path. */
pgb_status pgb_engine_autotune(pgb_engine *e, const pgb_prefs *prefs);
pgb_status pgb_engine_get_tuning(pgb_engine *e, int *threads, int *smem_windows);
pgb_status pgb_engine_set_tuning(pgb_engine *e, const int *threads, const int *smem_windows);

/* Device time of the last pgb_queries_run by phase, from CUDA events on the
 * engine's stream: [0] the stage-1 tensor-core contraction alone (part of
 * [2]), [1] stage-1 tables, [2] stage-1 scores and ranking, [3] stage-2
 * trials, [4] refinement and output; [5] total.
 * counts[0..7]: stage-1 (query, edge) pairs, stage-2 + refinement trials,
 * objective evaluations, site evaluations (both trial passes), stage-2 trials
 * launched, stage-2 trials consumed by the baseball stop rule, refinement
 * trials, baseball rounds. */
pgb_status pgb_engine_timings(pgb_engine *e, double *ms, double *counts);

#ifdef __cplusplus
}
#endif
#endif
