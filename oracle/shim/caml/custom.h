/* Test-infrastructure shim for <caml/custom.h>; see mlvalues.h. */
#ifndef PGPU_SHIM_CAML_CUSTOM_H
#define PGPU_SHIM_CAML_CUSTOM_H
#include "mlvalues.h"
struct custom_operations {
  const char *identifier;
  void (*finalize)(value v);
  int (*compare)(value v1, value v2);
  intptr_t (*hash)(value v);
  void (*serialize)(value v, unsigned long *bsize_32, unsigned long *bsize_64);
  unsigned long (*deserialize)(void *dst);
  int (*compare_ext)(value v1, value v2);
};
#define custom_hash_default        NULL
#define custom_compare_ext_default NULL
value caml_alloc_custom(struct custom_operations *ops, uintptr_t size,
                        uintptr_t mem, uintptr_t max);
void register_custom_operations(struct custom_operations *ops);
#endif
