/* Test-infrastructure shim for <caml/intext.h>; see mlvalues.h. */
#ifndef PGPU_SHIM_CAML_INTEXT_H
#define PGPU_SHIM_CAML_INTEXT_H
#include "mlvalues.h"
void caml_serialize_int_1(int i);
void caml_serialize_int_2(int i);
void caml_serialize_int_4(int32_t i);
void caml_serialize_int_8(int64_t i);
unsigned int caml_deserialize_uint_1(void);
unsigned int caml_deserialize_uint_2(void);
uint32_t caml_deserialize_uint_4(void);
uint64_t caml_deserialize_uint_8(void);
#endif
