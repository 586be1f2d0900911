/* Minimal stand-in for the OCaml runtime header of the same name, enough to
 * compile-check C stubs in a tree without an OCaml toolchain.  Test only. */
#ifndef SHIM_CAML_MLVALUES_H
#define SHIM_CAML_MLVALUES_H
#include <stdint.h>
typedef intptr_t value;
typedef uintptr_t mlsize_t;
#define CAMLprim
#define Val_unit ((value)1)
#define Val_int(x) ((value)(((intptr_t)(x) << 1) + 1))
#define Int_val(x) ((int)((x) >> 1))
#define Long_val(x) ((long)((x) >> 1))
#define Field(x, i) (((value *)(x))[i])
#define Wosize_val(x) (((uintptr_t *)(x))[-1] >> 10)
#define Double_flat_field(v, i) (((double *)(v))[i])
#define Double_val(v) (*(double *)(v))
#define Store_double_flat_field(v, i, d) (((double *)(v))[i] = (d))
#define Bytes_val(x) ((unsigned char *)(x))
#define Store_field(b, i, v) (Field(b, i) = (v))
#endif
