/* Test-infrastructure shim: definitions for the OCaml runtime hooks that
 * phylocaml's lib/bitvector/bv.c references from its OCaml-facing wrappers.
 * The oracle never calls those wrappers; every hook aborts if reached, so a
 * mistaken call cannot silently return garbage. */
#include <stdio.h>
#include <stdlib.h>
#include "caml/mlvalues.h"
#include "caml/custom.h"
#include "caml/intext.h"

static void shim_unreachable(const char *what)
{
  fprintf(stderr, "oracle shim: OCaml runtime hook %s called\n", what);
  abort();
}

uintptr_t pgpu_shim_wosize(value v) { (void)v; shim_unreachable("Wosize_val"); return 0; }
value caml_copy_int32(int32_t i) { (void)i; shim_unreachable("caml_copy_int32"); return 0; }
value caml_copy_int64(int64_t i) { (void)i; shim_unreachable("caml_copy_int64"); return 0; }
value caml_alloc(uintptr_t w, int t) { (void)w; (void)t; shim_unreachable("caml_alloc"); return 0; }
value caml_alloc_custom(struct custom_operations *o, uintptr_t s, uintptr_t m, uintptr_t x)
{ (void)o; (void)s; (void)m; (void)x; shim_unreachable("caml_alloc_custom"); return 0; }
void register_custom_operations(struct custom_operations *o) { (void)o; shim_unreachable("register_custom_operations"); }
void caml_serialize_int_1(int i) { (void)i; shim_unreachable("caml_serialize_int_1"); }
void caml_serialize_int_2(int i) { (void)i; shim_unreachable("caml_serialize_int_2"); }
void caml_serialize_int_4(int32_t i) { (void)i; shim_unreachable("caml_serialize_int_4"); }
void caml_serialize_int_8(int64_t i) { (void)i; shim_unreachable("caml_serialize_int_8"); }
unsigned int caml_deserialize_uint_1(void) { shim_unreachable("caml_deserialize_uint_1"); return 0; }
unsigned int caml_deserialize_uint_2(void) { shim_unreachable("caml_deserialize_uint_2"); return 0; }
uint32_t caml_deserialize_uint_4(void) { shim_unreachable("caml_deserialize_uint_4"); return 0; }
uint64_t caml_deserialize_uint_8(void) { shim_unreachable("caml_deserialize_uint_8"); return 0; }
/* lib/phyloc.c's Val_some, declared by lib/phyloc.h */
value Val_some(value v) { (void)v; shim_unreachable("Val_some"); return 0; }
