/* linear_gpu_stubs.c -- the OCaml C stubs of pplacer's Linear module
 * (pplacer_src/linear.ml:13-89) over the pplacer_gb300 GPU library.
 *
 * Replaces pplacer_src/linear_c.c in pplacer's C-side library: every
 * CAMLprim keeps the symbol name the OCaml `external` declaration binds,
 * reads the bigarray dimensions as linear_c.c does (the same printf warnings
 * on mismatched sizes, the same caml_failwith checks of
 * float_mat_int_vec_mul_c) and forwards plain pointers to the pgb_* entry
 * points of include/pplacer_gb300.h.  The OCaml sources, the CLI and the
 * jplace output stay unchanged; link with -lpplacer_gb300.
 *
 * Each call copies its operands to the GPU, runs one kernel and copies the
 * result back (FP64, the reference's arithmetic and summation order where
 * linear_c.c's is elementwise).  A GPU failure raises Failure with the
 * library's message instead of returning a wrong number.
 *
 * The print stubs (mat_print_c, ten_print_c) print on the host, as linear_c.c
 * does: they are debugging output, not numeric kernels.
 */
#include <stdint.h>
#include <stdio.h>

#include <caml/alloc.h>
#include <caml/bigarray.h>
#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>

#include "pplacer_gb300.h"

#define DATA(v) Caml_ba_data_val(v)
#define DIM(v, i) ((int)Caml_ba_array_val(v)->dim[i])

static void check_status(pgb_status s) {
  if (s != PGB_OK) caml_failwith(pgb_last_error());
}

/* A NaN from a likelihood entry point with an error message set is a GPU
 * failure; a NaN of the arithmetic itself (as linear_c.c can return) has no
 * message and passes through. */
static value box_result(double r) {
  if (r != r) {
    const char *msg = pgb_last_error();
    if (msg && msg[0]) caml_failwith(msg);
  }
  return caml_copy_double(r);
}

/* linear.ml:13 */
CAMLprim value gemmish_c(value dst, value a, value b) {
  CAMLparam3(dst, a, b);
  int n_states = DIM(a, 0), n_sites = DIM(b, 0);
  if (n_states != DIM(a, 1) || n_sites != DIM(dst, 0) || n_states != DIM(dst, 1)) printf("bad input dimensions!");
  check_status(pgb_gemmish(DATA(dst), DATA(a), DATA(b), n_sites, n_states));
  CAMLreturn(Val_unit);
}

/* linear.ml:19 */
CAMLprim value dediagonalize(value dst, value u, value lambda, value uit) {
  CAMLparam4(dst, u, lambda, uit);
  check_status(pgb_dediagonalize(DATA(dst), DATA(u), DATA(lambda), DATA(uit), DIM(lambda, 0)));
  CAMLreturn(Val_unit);
}

/* linear.ml:25 */
CAMLprim value mat_print_c(value x) {
  CAMLparam1(x);
  const double *p = DATA(x);
  int n_sites = DIM(x, 0), n_states = DIM(x, 1);
  for (int s = 0; s < n_sites; s++) {
    for (int k = 0; k < n_states; k++) printf("%g\t", *p++);
    printf("\n");
  }
  CAMLreturn(Val_unit);
}

/* linear.ml:28 */
CAMLprim value mat_log_like3_c(value statd, value x, value y, value z) {
  CAMLparam4(statd, x, y, z);
  CAMLreturn(box_result(pgb_mat_log_like3(DATA(statd), DATA(x), DATA(y), DATA(z), DIM(x, 0), DIM(x, 1))));
}

/* linear.ml:31 */
CAMLprim value mat_pairwise_prod_c(value dst, value x, value y) {
  CAMLparam3(dst, x, y);
  check_status(pgb_mat_pairwise_prod(DATA(dst), DATA(x), DATA(y), DIM(x, 0), DIM(x, 1)));
  CAMLreturn(Val_unit);
}

/* linear.ml:34 */
CAMLprim value mat_statd_pairwise_prod_c(value statd, value dst, value a, value b) {
  CAMLparam4(statd, dst, a, b);
  check_status(pgb_mat_statd_pairwise_prod(DATA(statd), DATA(dst), DATA(a), DATA(b), DIM(a, 0), DIM(a, 1)));
  CAMLreturn(Val_unit);
}

/* linear.ml:40 */
CAMLprim value mat_masked_logdot_c(value x, value y, value mask) {
  CAMLparam3(x, y, mask);
  if (DIM(x, 0) != DIM(mask, 0)) printf("mat_masked_logdot_c: Mask length doesn't match!");
  CAMLreturn(box_result(pgb_mat_masked_logdot(DATA(x), DATA(y), (const uint16_t *)DATA(mask), DIM(x, 0), DIM(x, 1))));
}

/* linear.ml:46 */
CAMLprim value mat_bounded_logdot_c(value x, value y, value first, value last) {
  CAMLparam4(x, y, first, last);
  CAMLreturn(box_result(
      pgb_mat_bounded_logdot(DATA(x), DATA(y), Int_val(first), Int_val(last), DIM(x, 0), DIM(x, 1))));
}

/* linear.ml:52 */
CAMLprim value ten_print_c(value x) {
  CAMLparam1(x);
  const double *p = DATA(x);
  int n_rates = DIM(x, 0), n_sites = DIM(x, 1), n_states = DIM(x, 2);
  for (int r = 0; r < n_rates; r++) {
    for (int s = 0; s < n_sites; s++) {
      for (int k = 0; k < n_states; k++) printf("%g\t", *p++);
      printf("\n");
    }
    printf("--\n");
  }
  CAMLreturn(Val_unit);
}

/* linear.ml:55 */
CAMLprim value ten_log_like3_c(value statd, value x, value y, value z, value util) {
  CAMLparam5(statd, x, y, z, util);
  CAMLreturn(box_result(pgb_ten_log_like3(DATA(statd), DATA(x), DATA(y), DATA(z), DATA(util), DIM(x, 0), DIM(x, 1),
                                          DIM(x, 2))));
}

/* linear.ml:58 */
CAMLprim value ten_pairwise_prod_c(value dst, value x, value y) {
  CAMLparam3(dst, x, y);
  check_status(pgb_ten_pairwise_prod(DATA(dst), DATA(x), DATA(y), DIM(x, 0), DIM(x, 1), DIM(x, 2)));
  CAMLreturn(Val_unit);
}

/* linear.ml:61 */
CAMLprim value ten_statd_pairwise_prod_c(value statd, value dst, value a, value b) {
  CAMLparam4(statd, dst, a, b);
  check_status(
      pgb_ten_statd_pairwise_prod(DATA(statd), DATA(dst), DATA(a), DATA(b), DIM(a, 0), DIM(a, 1), DIM(a, 2)));
  CAMLreturn(Val_unit);
}

/* linear.ml:67 */
CAMLprim value ten_masked_logdot_c(value x, value y, value mask, value util) {
  CAMLparam4(x, y, mask, util);
  if (DIM(x, 1) != DIM(mask, 0)) printf("ten_masked_logdot_c: Mask length doesn't match!");
  if (DIM(x, 1) != DIM(util, 0)) printf("ten_masked_logdot_c: Util length doesn't match!");
  CAMLreturn(box_result(pgb_ten_masked_logdot(DATA(x), DATA(y), (const uint16_t *)DATA(mask), DATA(util), DIM(x, 0),
                                              DIM(x, 1), DIM(x, 2))));
}

/* linear.ml:73 */
CAMLprim value ten_bounded_logdot_c(value x, value y, value first, value last, value util) {
  CAMLparam5(x, y, first, last, util);
  CAMLreturn(box_result(pgb_ten_bounded_logdot(DATA(x), DATA(y), Int_val(first), Int_val(last), DATA(util),
                                               DIM(x, 0), DIM(x, 1), DIM(x, 2))));
}

/* linear.ml:76 */
CAMLprim value vec_pairwise_prod_c(value dst, value x, value y) {
  CAMLparam3(dst, x, y);
  check_status(pgb_vec_pairwise_prod(DATA(dst), DATA(x), DATA(y), DIM(x, 0)));
  CAMLreturn(Val_unit);
}

/* linear.ml:80 */
CAMLprim value int_vec_tot_c(value x) {
  CAMLparam1(x);
  CAMLlocal1(tot);
  tot = Val_int(pgb_int_vec_tot((const uint16_t *)DATA(x), DIM(x, 0)));
  CAMLreturn(tot);
}

/* linear.ml:83 */
CAMLprim value int_vec_pairwise_prod_c(value dst, value x, value y) {
  CAMLparam3(dst, x, y);
  check_status(pgb_int_vec_pairwise_prod((uint16_t *)DATA(dst), (const uint16_t *)DATA(x),
                                         (const uint16_t *)DATA(y), DIM(dst, 0)));
  CAMLreturn(Val_unit);
}

/* linear.ml:89 */
CAMLprim value float_mat_int_vec_mul_c(value dst, value mat, value vec) {
  CAMLparam3(dst, mat, vec);
  int n = DIM(mat, 0), k = DIM(mat, 1);
  if (DIM(vec, 0) != n) caml_failwith("dim_0 vec != dim_0 mat");
  if (DIM(dst, 0) != k) caml_failwith("dim_0 dst != dim_1 mat");
  check_status(pgb_float_mat_int_vec_mul(DATA(dst), DATA(mat), (const uint16_t *)DATA(vec), n, k));
  CAMLreturn(Val_unit);
}
