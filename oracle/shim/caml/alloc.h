/* Test-infrastructure shim for <caml/alloc.h>; see mlvalues.h. */
#ifndef PGPU_SHIM_CAML_ALLOC_H
#define PGPU_SHIM_CAML_ALLOC_H
#include "mlvalues.h"
#endif
