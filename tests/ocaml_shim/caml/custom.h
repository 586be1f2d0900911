/* Minimal stand-in (test only). */
#ifndef SHIM_CAML_CUSTOM_H
#define SHIM_CAML_CUSTOM_H
#include "mlvalues.h"
struct custom_fixed_length;
struct custom_operations {
  const char *identifier;
  void (*finalize)(value v);
  int (*compare)(value v1, value v2);
  intptr_t (*hash)(value v);
  void (*serialize)(value v, uintptr_t *bsize_32, uintptr_t *bsize_64);
  uintptr_t (*deserialize)(void *dst);
  int (*compare_ext)(value v1, value v2);
  const struct custom_fixed_length *fixed_length;
};
#define custom_compare_default 0
#define custom_hash_default 0
#define custom_serialize_default 0
#define custom_deserialize_default 0
#define custom_compare_ext_default 0
#define custom_fixed_length_default 0
#define Data_custom_val(v) ((void *)&Field((v), 1))
#endif
