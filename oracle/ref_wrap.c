/* Plain-pointer wrappers around the reference's own pplacer_src/linear_c.c
 * (compiled unmodified against oracle/shim).  Each ref_* function builds the
 * bigarray descriptors the OCaml externals of pplacer_src/linear.ml:13-89
 * would pass and calls the CAMLprim symbol.  Layouts follow linear_c.c:6-12:
 * matrices are [site][state], tensors [rate][site][state], row-major.
 * Test infrastructure only (oracle/_ref): used by tests to pin the oracle's
 * restated kernels against the reference's arithmetic. */
#include <stdint.h>
#include "shim/caml/ocaml_shim.h"

value gemmish_c(value, value, value);
value dediagonalize(value, value, value, value);
value mat_log_like3_c(value, value, value, value);
value mat_pairwise_prod_c(value, value, value);
value mat_statd_pairwise_prod_c(value, value, value, value);
value mat_masked_logdot_c(value, value, value);
value mat_bounded_logdot_c(value, value, value, value);
value ten_log_like3_c(value, value, value, value, value);
value ten_pairwise_prod_c(value, value, value);
value ten_statd_pairwise_prod_c(value, value, value, value);
value ten_masked_logdot_c(value, value, value, value);
value ten_bounded_logdot_c(value, value, value, value, value);
value vec_pairwise_prod_c(value, value, value);
value int_vec_tot_c(value);
value int_vec_pairwise_prod_c(value, value, value);
value float_mat_int_vec_mul_c(value, value, value);

static struct caml_ba_array ba1(const void *p, long n0) {
  struct caml_ba_array b = {(void *)p, 1, 0, 0, {n0, 0, 0, 0}};
  return b;
}
static struct caml_ba_array ba2(const void *p, long n0, long n1) {
  struct caml_ba_array b = {(void *)p, 2, 0, 0, {n0, n1, 0, 0}};
  return b;
}
static struct caml_ba_array ba3(const void *p, long n0, long n1, long n2) {
  struct caml_ba_array b = {(void *)p, 3, 0, 0, {n0, n1, n2, 0}};
  return b;
}
#define V(b) ((value) & (b))
#define UNBOX(v) (*(double *)(v))

void ref_gemmish(double *dst, const double *a, const double *b, int n_sites, int n_states) {
  struct caml_ba_array d = ba2(dst, n_sites, n_states), A = ba2(a, n_states, n_states),
                       B = ba2(b, n_sites, n_states);
  gemmish_c(V(d), V(A), V(B));
}

void ref_dediagonalize(double *dst, const double *u, const double *lambda, const double *uit, int n) {
  struct caml_ba_array d = ba2(dst, n, n), U = ba2(u, n, n), L = ba1(lambda, n), W = ba2(uit, n, n);
  dediagonalize(V(d), V(U), V(L), V(W));
}

double ref_mat_log_like3(const double *statd, const double *x, const double *y, const double *z,
                         int n_sites, int n_states) {
  struct caml_ba_array s = ba1(statd, n_states), X = ba2(x, n_sites, n_states),
                       Y = ba2(y, n_sites, n_states), Z = ba2(z, n_sites, n_states);
  return UNBOX(mat_log_like3_c(V(s), V(X), V(Y), V(Z)));
}

void ref_mat_pairwise_prod(double *dst, const double *x, const double *y, int n_sites, int n_states) {
  struct caml_ba_array d = ba2(dst, n_sites, n_states), X = ba2(x, n_sites, n_states),
                       Y = ba2(y, n_sites, n_states);
  mat_pairwise_prod_c(V(d), V(X), V(Y));
}

void ref_mat_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                 int n_sites, int n_states) {
  struct caml_ba_array s = ba1(statd, n_states), d = ba2(dst, n_sites, n_states),
                       A = ba2(a, n_sites, n_states), B = ba2(b, n_sites, n_states);
  mat_statd_pairwise_prod_c(V(s), V(d), V(A), V(B));
}

double ref_mat_masked_logdot(const double *x, const double *y, const uint16_t *mask, int n_sites,
                             int n_states) {
  struct caml_ba_array X = ba2(x, n_sites, n_states), Y = ba2(y, n_sites, n_states),
                       M = ba1(mask, n_sites);
  return UNBOX(mat_masked_logdot_c(V(X), V(Y), V(M)));
}

double ref_mat_bounded_logdot(const double *x, const double *y, int first, int last, int n_sites,
                              int n_states) {
  struct caml_ba_array X = ba2(x, n_sites, n_states), Y = ba2(y, n_sites, n_states);
  return UNBOX(mat_bounded_logdot_c(V(X), V(Y), Val_int(first), Val_int(last)));
}

double ref_ten_log_like3(const double *statd, const double *x, const double *y, const double *z,
                         double *util, int n_rates, int n_sites, int n_states) {
  struct caml_ba_array s = ba1(statd, n_states), X = ba3(x, n_rates, n_sites, n_states),
                       Y = ba3(y, n_rates, n_sites, n_states), Z = ba3(z, n_rates, n_sites, n_states),
                       U = ba1(util, n_sites);
  return UNBOX(ten_log_like3_c(V(s), V(X), V(Y), V(Z), V(U)));
}

void ref_ten_pairwise_prod(double *dst, const double *x, const double *y, int n_rates, int n_sites,
                           int n_states) {
  struct caml_ba_array d = ba3(dst, n_rates, n_sites, n_states), X = ba3(x, n_rates, n_sites, n_states),
                       Y = ba3(y, n_rates, n_sites, n_states);
  ten_pairwise_prod_c(V(d), V(X), V(Y));
}

void ref_ten_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                 int n_rates, int n_sites, int n_states) {
  struct caml_ba_array s = ba1(statd, n_states), d = ba3(dst, n_rates, n_sites, n_states),
                       A = ba3(a, n_rates, n_sites, n_states), B = ba3(b, n_rates, n_sites, n_states);
  ten_statd_pairwise_prod_c(V(s), V(d), V(A), V(B));
}

double ref_ten_masked_logdot(const double *x, const double *y, const uint16_t *mask, double *util,
                             int n_rates, int n_sites, int n_states) {
  struct caml_ba_array X = ba3(x, n_rates, n_sites, n_states), Y = ba3(y, n_rates, n_sites, n_states),
                       M = ba1(mask, n_sites), U = ba1(util, n_sites);
  return UNBOX(ten_masked_logdot_c(V(X), V(Y), V(M), V(U)));
}

double ref_ten_bounded_logdot(const double *x, const double *y, int first, int last, double *util,
                              int n_rates, int n_sites, int n_states) {
  struct caml_ba_array X = ba3(x, n_rates, n_sites, n_states), Y = ba3(y, n_rates, n_sites, n_states),
                       U = ba1(util, n_sites);
  return UNBOX(ten_bounded_logdot_c(V(X), V(Y), Val_int(first), Val_int(last), V(U)));
}

void ref_vec_pairwise_prod(double *dst, const double *x, const double *y, int n) {
  struct caml_ba_array d = ba1(dst, n), X = ba1(x, n), Y = ba1(y, n);
  vec_pairwise_prod_c(V(d), V(X), V(Y));
}

int ref_int_vec_tot(const uint16_t *x, int n) {
  struct caml_ba_array X = ba1(x, n);
  return Int_val(int_vec_tot_c(V(X)));
}

void ref_int_vec_pairwise_prod(uint16_t *dst, const uint16_t *x, const uint16_t *y, int n) {
  struct caml_ba_array d = ba1(dst, n), X = ba1(x, n), Y = ba1(y, n);
  int_vec_pairwise_prod_c(V(d), V(X), V(Y));
}

void ref_float_mat_int_vec_mul(double *dst, const double *mat, const uint16_t *vec, int n, int k) {
  struct caml_ba_array d = ba1(dst, k), M = ba2(mat, n, k), X = ba1(vec, n);
  float_mat_int_vec_mul_c(V(d), V(M), V(X));
}
