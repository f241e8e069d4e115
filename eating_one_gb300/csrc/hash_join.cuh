// hash_join.cuh - table build and probe building blocks shared by the hash
// join, the single-hash join, the hash and sort indexes, the left outer join
// and the star join.
#pragma once

#include <algorithm>

#include "ej_internal.h"

struct ej_table_plan_t {
  int kind = EJ_TABLE_HASH;
  uint64_t nR = 0;
  uint32_t hb = 1;      // key bits sorted on (bucket bits; 32 for a sorted index)
  uint32_t passes = 1;  // LSD radix passes
  uint32_t nfence = 0;  // sorted index: fence entries
  size_t rs_off = 0, start_off = 0, tmp_off = 0;  // arena offsets (rs/start unused with own storage)
  ej_radix_plan rplan;
};

struct ej_probe_plan_t {
  uint64_t nP = 0;
  uint64_t ntiles = 0;
  size_t count_off = 0, off_off = 0, scan_off = 0;
};

struct ej_probe_layout {
  uint32_t pb = 0;  // partition bits of the probe side (0 = probe in place)
  ej_radix_plan splan;
  size_t spart_off = 0;
  ej_probe_plan_t pp;
};

size_t ej_table_bytes(uint64_t nR, int delta = 0);
void ej_table_plan(ej_plan_bytes& p, ej_table_plan_t& tp, uint64_t nR, bool own_storage, int kind, int delta = 0);
// aux: bucket starts (hash, 2^hb+1 uint32) or fence (sorted, nfence int32)
ej_status ej_table_build(ej_handle* h, const ej_table_plan_t& tp, const ej_tuple* R, ej_tuple* rs, void* aux,
                         ej_table_view* view);

uint64_t ej_probe_tiles(uint64_t nP);
void ej_probe_plan(ej_plan_bytes& p, ej_probe_plan_t& pp, uint64_t nP);
// count pass + scan; the total goes to *d_count (device) when d_count != nullptr
ej_status ej_probe_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, unsigned long long* d_count);
// write pass; needs the offsets of ej_probe_count from the same plan
ej_status ej_probe_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, ej_result* out, uint64_t cap);

uint32_t ej_probe_partition_bits(const ej_handle* h, uint64_t nR, uint64_t nS);
void ej_probe_layout_add(ej_plan_bytes& p, ej_probe_layout& L, uint64_t nS, uint32_t pb);
ej_status ej_probe_exec(ej_handle* h, const ej_probe_layout& L, const ej_table_view& t, const ej_tuple* S,
                        bool outer, bool count_only, ej_result* out, uint64_t out_cap,
                        unsigned long long* d_count);

// mode: 0 = partition S when the planner says so, 1 = never partition S, 2 = count only
ej_status ej_hash_join_run(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                           ej_result* out, uint64_t out_cap, unsigned long long* d_count, int mode);
