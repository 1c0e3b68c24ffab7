/* Minimal stand-in for the OCaml runtime's value macros, written for this
 * project so that the reference's plain-C BEM stubs (src/bem3d_stubs.c) can
 * be compiled unmodified and driven from C.  TEST INFRASTRUCTURE ONLY: used
 * by oracle/ref_bem_harness.c to produce reference BEM matrices.
 *
 * Only what bem3d_stubs.c uses is defined.  A block is laid out as in OCaml's
 * heap: one header word holding the block's size in words, then the fields;
 * a value is the address of the first field.  Float arrays hold their
 * doubles directly (one word each on a 64-bit host); boxed doubles are a
 * pointer to one double.  There is no garbage collector, so the
 * registration macros do nothing. */
#ifndef NMAG_CAML_SHIM_MLVALUES_H
#define NMAG_CAML_SHIM_MLVALUES_H
#include <stdint.h>

typedef intptr_t value;

#define CAMLprim
#define Val_unit ((value)1)
#define Wosize_val(v) ((uintptr_t)(((const value *)(v))[-1]))
#define Field(v, i) (((value *)(v))[i])
#define Double_val(v) (*(const double *)(v))
#define Double_field(v, i) (((const double *)(v))[i])
#define Store_double_field(v, i, d) (((double *)(v))[i] = (d))

#endif
