/* Minimal stand-in (test only). */
#ifndef SHIM_CAML_ALLOC_H
#define SHIM_CAML_ALLOC_H
#include "mlvalues.h"
struct custom_operations;
value caml_alloc(mlsize_t wosize, int tag);
value caml_alloc_tuple(mlsize_t wosize);
value caml_alloc_float_array(mlsize_t len);
value caml_copy_double(double d);
value caml_alloc_custom(struct custom_operations *ops, uintptr_t size, mlsize_t mem,
                        mlsize_t max);
#endif
