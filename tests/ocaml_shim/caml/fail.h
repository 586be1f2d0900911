/* Minimal stand-in (test only). */
#ifndef SHIM_CAML_FAIL_H
#define SHIM_CAML_FAIL_H
#include "mlvalues.h"
void caml_failwith(const char *msg);
void caml_raise_constant(value tag);
#endif
