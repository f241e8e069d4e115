// onesweep.cuh - LSD radix sort with one scatter launch per digit (onesweep.cu).
#pragma once

#include "ej_internal.h"

struct ej_onesweep_plan {
  uint64_t n = 0;
  uint32_t ntiles = 0;
  size_t hist_off = 0, base_off = 0, status_off = 0, ctr_off = 0;
  size_t status_bytes = 0;
};

void ej_onesweep_plan_add(ej_plan_bytes& p, ej_onesweep_plan& op, uint64_t n);
// R (n rows) ordered by the order key of digit_kind (EJ_DIGIT_HASH: hash32(val);
// EJ_DIGIT_VALUE: val as signed) into the columns rkey/rval; tmp_a and tmp_b
// hold n tuples each
ej_status ej_onesweep_sort(ej_handle* h, const ej_onesweep_plan& op, const ej_tuple* R, ej_tuple* tmp_a,
                           ej_tuple* tmp_b, int32_t* rkey, int32_t* rval, int digit_kind);
