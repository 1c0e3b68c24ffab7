/* Minimal stand-in (see mlvalues.h): no garbage collector, so registering
 * parameters and locals only declares the locals. */
#ifndef NMAG_CAML_SHIM_MEMORY_H
#define NMAG_CAML_SHIM_MEMORY_H
#include "mlvalues.h"

#define CAMLparam2(a, b) ((void)(a), (void)(b))
#define CAMLlocal3(a, b, c) value a = 0, b = 0, c = 0
#define CAMLreturn(x) return (x)

#endif
