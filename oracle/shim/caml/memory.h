/* Test-infrastructure shim for <caml/memory.h>: the GC root macros become
 * plain local declarations (no GC exists in the oracle). */
#ifndef PGPU_SHIM_CAML_MEMORY_H
#define PGPU_SHIM_CAML_MEMORY_H
#include "mlvalues.h"
#define CAMLparam0()                 do { } while (0)
#define CAMLparam1(a)                (void)(a)
#define CAMLparam2(a, b)             ((void)(a), (void)(b))
#define CAMLparam3(a, b, c)          ((void)(a), (void)(b), (void)(c))
#define CAMLparam4(a, b, c, d)       ((void)(a), (void)(b), (void)(c), (void)(d))
#define CAMLlocal1(a)                value a = Val_unit
#define CAMLlocal2(a, b)             value a = Val_unit, b = Val_unit
#define CAMLreturn(x)                return (x)
#endif
