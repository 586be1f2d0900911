/* Minimal stand-in (test only). */
#ifndef SHIM_CAML_CALLBACK_H
#define SHIM_CAML_CALLBACK_H
#include "mlvalues.h"
const value *caml_named_value(const char *name);
#endif
