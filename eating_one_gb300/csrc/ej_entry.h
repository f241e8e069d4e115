// ej_entry.h - helpers shared by the C ABI entry points of every translation unit.
#pragma once

#include "ej_internal.h"

// clear the last error and make the handle's device current
ej_status ej_begin(ej_handle* h);
// synchronise the stream; *count <- device word d_words[0]; device errors other
// than EJ_ERR_CAPACITY are returned (and the status word is cleared)
ej_status ej_finish(ej_handle* h, uint64_t* count);
ej_status ej_check_rel(ej_handle* h, const char* name, const ej_tuple* p, uint64_t n);
ej_status ej_check_out(ej_handle* h, const void* out, uint64_t cap, const uint64_t* out_count);
ej_status ej_capacity_result(ej_handle* h, uint64_t count, uint64_t cap);
