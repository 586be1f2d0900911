/* Minimal stand-in (test only): the local-root macros reduce to no-ops. */
#ifndef SHIM_CAML_MEMORY_H
#define SHIM_CAML_MEMORY_H
#include "mlvalues.h"
#define CAMLparam1(a) (void)(a)
#define CAMLparam2(a, b) ((void)(a), (void)(b))
#define CAMLparam4(a, b, c, d) ((void)(a), (void)(b), (void)(c), (void)(d))
#define CAMLparam5(a, b, c, d, e) ((void)(a), (void)(b), (void)(c), (void)(d), (void)(e))
#define CAMLxparam1(a) (void)(a)
#define CAMLxparam2(a, b) ((void)(a), (void)(b))
#define CAMLxparam5(a, b, c, d, e) ((void)(a), (void)(b), (void)(c), (void)(d), (void)(e))
#define CAMLlocal1(a) value a = Val_unit
#define CAMLlocal4(a, b, c, d) value a = Val_unit, b = Val_unit, c = Val_unit, d = Val_unit
#define CAMLreturn(x) return (x)
#endif
