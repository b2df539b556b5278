/* Minimal stand-in for the few OCaml runtime names that pplacer's
 * pplacer_src/linear_c.c uses, so that file compiles unmodified into a plain C
 * library for the oracle.  A "value" is a pointer to a bigarray descriptor
 * (struct caml_ba_array) or a tagged integer; boxed doubles are returned
 * through a thread-local slot that the caller reads immediately.
 * Test infrastructure only: never linked into the product. */
#ifndef ORACLE_OCAML_SHIM_H
#define ORACLE_OCAML_SHIM_H
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

typedef intptr_t value;
typedef intptr_t intnat;

struct caml_ba_array {
  void *data;
  intnat num_dims;
  intnat flags;
  void *proxy;
  intnat dim[4];
};

#define CAMLprim
#define CAMLparam0()
#define CAMLparam1(a) (void)(a)
#define CAMLparam2(a, b) (void)(a); (void)(b)
#define CAMLparam3(a, b, c) (void)(a); (void)(b); (void)(c)
#define CAMLparam4(a, b, c, d) (void)(a); (void)(b); (void)(c); (void)(d)
#define CAMLparam5(a, b, c, d, e) (void)(a); (void)(b); (void)(c); (void)(d); (void)(e)
#define CAMLlocal1(x) value x = 0
#define CAMLreturn(x) return (x)

#define Caml_ba_array_val(v) ((struct caml_ba_array *)(v))
#define Caml_ba_data_val(v) (Caml_ba_array_val(v)->data)
#define Int_val(v) ((int)(((intnat)(v)) >> 1))
#define Val_int(x) ((value)((((intnat)(x)) << 1) + 1))
#define Val_unit Val_int(0)

static __thread double oracle_shim_double_box;
static inline value caml_copy_double(double d) {
  oracle_shim_double_box = d;
  return (value)&oracle_shim_double_box;
}
static inline void caml_failwith(const char *msg) {
  fprintf(stderr, "caml_failwith: %s\n", msg);
  abort();
}
#endif
