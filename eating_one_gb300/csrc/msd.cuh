// msd.cuh - the MSD table build of large hash tables (msd.cu).
#pragma once

#include "ej_internal.h"

// Hash tables of at least this many rows are sorted by two unordered MSD
// passes and a per-bucket shared-memory sort (msd.cu); smaller ones by the
// LSD passes, whose few tiles cost less than 65536 bucket sorts.
constexpr uint64_t EJ_MSD_MIN_ROWS = 1ull << 20;

struct ej_msd_plan {
  uint64_t n = 0;
  ej_radix_plan pass1;  // by hash bits 24..31, uniform tiles
  ej_radix_plan pass2;  // by bits 16..23, device-described tiles (at most one more per segment)
  size_t desc_off = 0, seg_off = 0, bstart_off = 0;
};

void ej_msd_plan_add(ej_plan_bytes& p, ej_msd_plan& mp, uint64_t n);
// R (n rows) ordered by hash32(val) into the columns rkey/rval (n rows each);
// tmp_a and tmp_b hold n tuples each
ej_status ej_msd_sort(ej_handle* h, const ej_msd_plan& mp, const ej_tuple* R, ej_tuple* tmp_a, ej_tuple* tmp_b,
                      int32_t* rkey, int32_t* rval);
