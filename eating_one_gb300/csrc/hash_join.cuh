// hash_join.cuh - table build and probe building blocks shared by the hash
// join, the single-hash join, the hash and sort indexes, the left outer join
// and the star join.
#pragma once

#include <algorithm>

#include "ej_internal.h"
#include "msd.cuh"
#include "onesweep.cuh"

// Hash tables of at least EJ_DIR_MIN_ROWS rows may carry a key directory (one
// load per probe, seven build launches): the build keeps it when the table's
// runs average two rows or more and otherwise switches to bucket bounds (one
// build launch); tables from EJ_DIR_PROBE_MIN_ROWS rows keep it whenever the
// caller probes 16 rows per table row or more.  Smaller tables carry bucket
// bounds (the bucket scan costs no more than a directory lookup while the
// table sits in L2).
constexpr uint64_t EJ_DIR_MIN_ROWS = 1ull << 22;
constexpr uint64_t EJ_DIR_PROBE_MIN_ROWS = 1ull << 20;
// a sorted table's aux storage: the value buckets' header, then the bounds
constexpr size_t EJ_VBUCKET_HEADER_BYTES = 256;

struct ej_table_plan_t {
  int kind = EJ_TABLE_HASH;
  bool use_dir = false;     // hash tables: key directory (else bucket bounds), unless the build
                            // finds short runs and no probe-heavy caller (then bucket bounds too)
  bool prefer_dir = false;  // the caller probes 16 or more rows per table row: keep the directory
  uint64_t nR = 0;
  uint32_t hb = 1;      // bucket bits (hash buckets, or value buckets of a sorted table)
  uint32_t passes = 4;  // LSD radix passes over the 32-bit key
  bool msd = false;       // large hash tables: MSD passes + bucket sorts instead (msd.cuh)
  ej_msd_plan mplan;
  bool onesweep = false;  // sorted indexes (and hash tables when chosen): one scatter launch per digit
  ej_onesweep_plan oplan;
  // arena offsets; rkey/rval/aux are unused when the table has its own storage
  size_t rkey_off = 0, rval_off = 0, aux_off = 0, tmp_a_off = 0, tmp_b_off = 0;
  // key directory build scratch (hash tables)
  size_t dir_keys_off = 0, dir_off_off = 0, dir_scan_off = 0, dir_kmax_off = 0, dir_kpre_off = 0;
  ej_radix_plan rplan;
};

struct ej_probe_plan_t {
  uint64_t nP = 0;
  uint32_t warps = 8;    // warps (128-probe warp tiles) per block
  uint64_t ntiles = 0;   // blocks of 128 * warps probes
  uint64_t nwtiles = 0;  // warp tiles of 128 probes
  size_t count_off = 0, off_off = 0, scan_off = 0;
  bool with_desc = false;  // run descriptors for the write pass
  size_t desc_off = 0;
};

struct ej_probe_layout {
  uint32_t pb = 0;  // partition bits of the probe side (0 = probe in place)
  ej_radix_plan splan;
  size_t spart_off = 0;
  ej_probe_plan_t pp;
};

size_t ej_table_bytes(uint64_t nR, int delta = 0);
// bytes of one column (rkey or rval) including the vector-load padding
size_t ej_table_col_bytes(uint64_t nR);
// bytes of the bucket bounds or the key directory (hash), or the value
// buckets and their header (sorted)
size_t ej_table_aux_bytes(const ej_table_plan_t& tp);
// the tuned choices of a table's build (bucket-bits delta, EJ_BUILD_*,
// EJ_TABLE_FORMAT_*; 0 in the last two: the planner's)
struct ej_table_knobs {
  int delta = 0;
  int build = EJ_BUILD_PLANNER;
  int table = EJ_TABLE_FORMAT_PLANNER;
};
ej_table_knobs ej_tuned_table_knobs(const ej_handle* h, uint64_t nR);
// n_probe: the probe rows the caller expects (0: unknown)
void ej_table_plan(ej_plan_bytes& p, ej_table_plan_t& tp, uint64_t nR, bool own_storage, int kind,
                   const ej_table_knobs& k = ej_table_knobs(), uint64_t n_probe = 0);
ej_status ej_table_build(ej_handle* h, const ej_table_plan_t& tp, const ej_tuple* R, int32_t* rkey, int32_t* rval,
                         void* aux, ej_table_view* view);

void ej_probe_plan(ej_plan_bytes& p, ej_probe_plan_t& pp, uint64_t nP, bool with_desc, uint32_t warps = 8);
// count pass (storing run descriptors when planned with them) + scan of the
// warp-tile totals; the total goes to *d_count (device) when d_count != nullptr
ej_status ej_probe_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, unsigned long long* d_count);
// write pass from the run descriptors and offsets of ej_probe_count (same
// plan, same inputs, same outer flag)
ej_status ej_probe_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         ej_result* out, uint64_t cap, bool outer = false);

uint32_t ej_probe_partition_bits(const ej_handle* h, uint64_t nR, uint64_t nS);
// two_pass: plan the run descriptors of ej_probe_count + ej_probe_write (for
// callers that read the count in between); ej_probe_exec needs none
void ej_probe_layout_add(ej_plan_bytes& p, ej_probe_layout& L, uint64_t nS, uint32_t pb, bool count_only,
                         bool two_pass = false, uint32_t warps = 8);
ej_status ej_probe_exec(ej_handle* h, const ej_probe_layout& L, const ej_table_view& t, const ej_tuple* S,
                        bool outer, bool count_only, ej_result* out, uint64_t out_cap,
                        unsigned long long* d_count);

// What a hash-join count leaves in the handle's arena for the write that
// follows it: the table, the probe side as probed (S or its partitioned
// copy) and the probe layout with its run descriptors and warp-tile offsets.
struct ej_prepared_join {
  const ej_tuple* R = nullptr;
  uint64_t nR = 0;
  const ej_tuple* S = nullptr;
  uint64_t nS = 0;
  const void* arena = nullptr;  // the arena allocation the state lives in
  const ej_tuple* P = nullptr;  // the probes the count walked
  ej_probe_layout L;
  ej_table_view t;
  bool count_known = false;  // the count reached the host (synchronous count call)
  uint64_t count = 0;
};

// mode: 0 = partition S when the planner says so, 1 = never partition S, 2 = count only
ej_status ej_hash_join_run(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                           ej_result* out, uint64_t out_cap, unsigned long long* d_count, int mode);
