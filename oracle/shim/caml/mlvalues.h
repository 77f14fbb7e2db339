/* Test-infrastructure shim: the smallest subset of the OCaml runtime's
 * <caml/mlvalues.h> that lets phylocaml's lib/bitvector/bv.c compile as a
 * plain C library.  The oracle calls only the pure C routines of bv.c
 * (bv_fitch, bv_distance, bv_union, bv_inter, bv_copy); the OCaml-facing
 * wrappers are compiled but never called, so their runtime hooks below are
 * stubs that abort.  Not part of the product. */
#ifndef PGPU_SHIM_CAML_MLVALUES_H
#define PGPU_SHIM_CAML_MLVALUES_H
#include <stdint.h>
#include <stddef.h>

typedef intptr_t value;

#define CAMLprim
#define CAMLextern extern

#define Val_long(x)           ((value)((((intptr_t)(x)) << 1) + 1))
#define Long_val(x)           (((intptr_t)(x)) >> 1)
#define Val_int(x)            Val_long(x)
#define Int_val(x)            ((int)Long_val(x))
#define Unsigned_long_val(x)  (((uintptr_t)(x)) >> 1)
#define Unsigned_int_val(x)   ((unsigned int)Unsigned_long_val(x))
#define Val_unit              Val_int(0)
#define Val_emptylist         Val_int(0)
#define Field(x, i)           (((value *)(x))[i])
#define Store_field(b, i, v)  (Field(b, i) = (v))
#define Int32_val(v)          (*(int32_t *)(v))
#define Int64_val(v)          (*(int64_t *)(v))
#define Double_val(v)         (*(double *)(v))
#define Data_custom_val(v)    ((void *)&Field((v), 1))
#define Wosize_val(v)         (pgpu_shim_wosize(v))

uintptr_t pgpu_shim_wosize(value v);
value caml_copy_int32(int32_t i);
value caml_copy_int64(int64_t i);
value caml_alloc(uintptr_t wosize, int tag);
#endif
