// probe.cuh - where a probe value's matches lie in a table (device code).
//
// A table stores R as rkey[]/rval[] in one order (ej_table_view).  In both
// kinds the matches of a value v form one contiguous run [lo, lo + c):
//   EJ_TABLE_HASH    rows sorted by hash32(val).  Single tables of 2^22 rows
//                    or more whose runs average two rows or more, and those
//                    of 2^20 rows or more whose caller probes 16 rows per
//                    table row, carry a key directory (8-byte entries {hash, lo} in hash order,
//                    linear probing from slot hash >> (32 - bits), each slot
//                    holding the first key at or after it, so c is the next
//                    slot's start minus lo); the others, smaller and batched
//                    tables carry bucket bounds: the run lies inside bucket b
//                    = top hb hash bits, rows [bucket[b].x, bucket[b].y) (one
//                    8-byte load);
//   EJ_TABLE_SORTED  rows sorted by val, with bucket bounds over value
//                    prefixes: bucket b = (v - vmin) >> vshift (the table's
//                    smallest and largest vals and the shift in a small
//                    device header, EjValueBuckets).
// A bucket is scanned with two 16-byte loads of rval (8 values), then 4
// values per round; in a sorted table a run or a bucket still open after two
// rounds is finished by binary search on the table's order key.
#pragma once

#include "ej_device.cuh"

__device__ __forceinline__ uint32_t ej_bucket_of(int32_t val, uint32_t hb) {
  return ej_hash32((uint32_t)val) >> (32u - hb);
}

// the value buckets of a sorted table: every row's val lies in [vmin, vmax];
// bucket of v = (v - vmin) >> vshift, below 2^hb (vmin > vmax: no rows)
struct EjValueBuckets {
  int32_t vmin, vmax;
  uint32_t vshift, pad;
};

// the order of a table's rows: hash32(val) (hash tables), val as an unsigned
// order-preserving key (sorted tables)
template <int KIND>
__device__ __forceinline__ uint32_t ej_order_key(int32_t v) {
  return KIND == 0 ? ej_hash32((uint32_t)v) : ((uint32_t)v ^ 0x80000000u);
}

struct EjHashBucketOf {
  uint32_t hb;
  __device__ __forceinline__ int32_t operator()(int32_t v) const { return (int32_t)ej_bucket_of(v, hb); }
};
struct EjValueBucketOf {
  int32_t vmin;
  uint32_t vshift;
  __device__ __forceinline__ int32_t operator()(int32_t v) const {
    return (int32_t)(((uint32_t)v - (uint32_t)vmin) >> vshift);
  }
};

// Table build: bucket b begins at row i, so bucket[b].x = i (b < nb) and the
// previous bucket ends there, bucket[b - 1].y = i (b > 0).
__device__ __forceinline__ void ej_set_bucket_begin(uint2* bucket, int64_t b, int64_t nb, uint32_t i) {
  uint32_t* w = reinterpret_cast<uint32_t*>(bucket);
  if (b < nb) w[2 * b] = i;
  if (b > 0) w[2 * b - 1] = i;
}

// Table build, one warp: the bounds of the 2^hb buckets that begin at rows
// [r0, r0 + 256) of a column of n rows in bucket order (bucket_of is
// non-decreasing along it); row n (when in range) is the end, which begins
// the buckets past the last row's.  Lane l looks at rows r0 + 32k + l
// (coalesced loads, all issued together) and takes the bucket of the row
// before from its neighbour lane.
template <class BucketOf>
__device__ __forceinline__ void ej_bucket_bounds_warp(const int32_t* __restrict__ rval, uint64_t n, uint64_t r0,
                                                      uint32_t hb, uint2* __restrict__ bucket, BucketOf bucket_of) {
  const unsigned int lane = threadIdx.x & 31u;
  const int32_t nb = (int32_t)(1u << hb);
  int32_t cur[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint64_t i = r0 + (uint64_t)k * 32 + lane;
    cur[k] = i < n ? bucket_of(rval[i]) : nb;
  }
  int32_t carry = -1;  // bucket of row r0 + 32k - 1
  if (r0 > 0) carry = r0 - 1 < n ? bucket_of(rval[r0 - 1]) : nb;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int32_t up = __shfl_up_sync(EJ_FULL_MASK, cur[k], 1);
    const int32_t prev = lane == 0 ? carry : up;
    carry = __shfl_sync(EJ_FULL_MASK, cur[k], 31);
    const uint64_t i = r0 + (uint64_t)k * 32 + lane;
    // a long run of empty buckets (a heavily duplicated key) is filled by the
    // whole warp, the rest by each lane
    const bool wide = i <= n && cur[k] - prev > 32;
    if (i <= n && !wide)
      for (int32_t b = prev + 1; b <= cur[k]; b++) ej_set_bucket_begin(bucket, b, nb, (uint32_t)i);
    for (unsigned int m = __ballot_sync(EJ_FULL_MASK, wide); m; m &= m - 1u) {
      const int src = __ffs(m) - 1;
      const int32_t p = __shfl_sync(EJ_FULL_MASK, prev, src), c = __shfl_sync(EJ_FULL_MASK, cur[k], src);
      const uint32_t row = (uint32_t)__shfl_sync(EJ_FULL_MASK, (unsigned long long)i, src);
      for (int32_t b = p + 1 + (int32_t)lane; b <= c; b += 32) ej_set_bucket_begin(bucket, b, nb, row);
    }
  }
}

// N binary searches advancing together, one load each per round: for every
// j with bit j of `active` (whose range must not be empty: lo[j] < hi[j]),
// the first index in [lo[j], hi[j]) whose row's order key is above key[j]
// (upper) or at least key[j] (lower), into lo[j]; hi[j] when there is none
template <int KIND, int N>
__device__ __forceinline__ void ej_search_rows(const int32_t* __restrict__ rv, uint32_t active, bool upper,
                                               const uint32_t (&key)[N], uint32_t (&lo)[N], uint32_t (&hi)[N]) {
  while (active) {
    int32_t x[N];
    uint32_t mid[N];
#pragma unroll
    for (int j = 0; j < N; j++)
      if (active & (1u << j)) {
        mid[j] = lo[j] + ((hi[j] - lo[j]) >> 1);
        x[j] = __ldg(rv + mid[j]);
      }
#pragma unroll
    for (int j = 0; j < N; j++) {
      if (!(active & (1u << j))) continue;
      const uint32_t k = ej_order_key<KIND>(x[j]);
      if (upper ? k <= key[j] : k < key[j]) lo[j] = mid[j] + 1; else hi[j] = mid[j];
      if (lo[j] >= hi[j]) active &= ~(1u << j);
    }
  }
}

constexpr int EJ_SCAN_ROUNDS = 2;  // linear rounds of 4 values past a bucket's first 8

// Runs of N probe values at once through bucket bounds (hash tables without
// a directory, and sorted tables): the bounds of every value's bucket, then
// the bucket's first 8 values (two 16-byte loads) for every value; a run or
// a bucket that goes on past them continues 4 values per round (sorted
// tables: for up to EJ_SCAN_ROUNDS rounds, then by binary search), all N
// advancing together.  ok[j] false: c[j] = 0.
template <int KIND, int N>
__device__ __forceinline__ void ej_find_runs_bucket(const ej_table_view& t, const int32_t (&v)[N],
                                                    const bool (&ok)[N], uint32_t (&lo)[N], uint32_t (&c)[N]) {
  uint32_t s0[N], s1[N];
  EjValueBuckets vb = {1, 0, 0u, 0u};
  if (KIND != 0) {
    const uint4 h = __ldg(reinterpret_cast<const uint4*>(t.vbuckets));
    vb.vmin = (int32_t)h.x;
    vb.vmax = (int32_t)h.y;
    vb.vshift = h.z;
  }
#pragma unroll
  for (int j = 0; j < N; j++) {
    s0[j] = s1[j] = 0;
    if (KIND == 0 && ok[j]) {
      const uint2 bb = __ldg(t.bucket + ej_bucket_of(v[j], t.hb));
      s0[j] = bb.x;
      s1[j] = bb.y;
    } else if (KIND != 0 && ok[j] && v[j] >= vb.vmin && v[j] <= vb.vmax) {
      const uint2 bb = __ldg(t.bucket + (((uint32_t)v[j] - (uint32_t)vb.vmin) >> vb.vshift));
      s0[j] = bb.x;
      s1[j] = bb.y;
    }
  }
  // vector loads address the aligned base rval - voff; positions are shifted
  // by voff while scanning and shifted back when recorded
  const int4* rv4 = reinterpret_cast<const int4*>(t.rval - t.voff);
#pragma unroll
  for (int j = 0; j < N; j++) {
    s0[j] += t.voff;
    s1[j] += t.voff;
  }
  int4 qa[N], qb[N];
#pragma unroll
  for (int j = 0; j < N; j++) {
    qa[j] = qb[j] = make_int4(0, 0, 0, 0);
    const uint32_t base = s0[j] & ~3u;
    if (s0[j] < s1[j]) {
      qa[j] = __ldg(rv4 + base / 4);
      if (base + 4 < s1[j]) qb[j] = __ldg(rv4 + base / 4 + 1);
    }
  }
  uint32_t upper = 0, lower = 0;  // bit j: the run (upper) or the search (lower) of probe j goes on past the 8
  uint32_t key[N], sl[N], sh[N];
#pragma unroll
  for (int j = 0; j < N; j++) {
    // equality mask of the 8 loaded values, restricted to the bucket
    const uint32_t base = s0[j] & ~3u;
    const int x[8] = {qa[j].x, qa[j].y, qa[j].z, qa[j].w, qb[j].x, qb[j].y, qb[j].z, qb[j].w};
    uint32_t eq = 0;
#pragma unroll
    for (int e = 0; e < 8; e++) eq |= (x[e] == v[j] ? 1u : 0u) << e;
    const uint32_t from = s0[j] - base;                            // 0..3
    const uint32_t to = s1[j] - base < 8u ? s1[j] - base : 8u;     // end of the bucket within the 8
    eq &= ((1u << to) - 1u) & ~((1u << from) - 1u);
    // rows are in order-key order, so the matches are one contiguous run
    c[j] = __popc(eq);
    lo[j] = c[j] ? base + (uint32_t)(__ffs(eq) - 1) : s1[j];
    key[j] = ej_order_key<KIND>(v[j]);
    sl[j] = base + 8;
    sh[j] = s1[j];
    // a run goes on past the 8 loaded values only if it reaches their end; with
    // no match yet, the search goes on only if the bucket does
    if (sl[j] < sh[j]) {
      if (c[j] && (eq & 0x80u)) upper |= 1u << j;
      else if (!c[j] && to >= 8u) lower |= 1u << j;
    }
  }
  const int32_t* rv = t.rval - t.voff;
  // 4 more values per round (one 16-byte load per probe and round): hash
  // tables until the run or the bucket ends (a long run there is a key with
  // many rows in a small table); sorted tables, whose value buckets can be
  // wide, for up to EJ_SCAN_ROUNDS rounds, then by binary search
  uint32_t more = upper | lower;
#pragma unroll 1
  for (int r = 0; (KIND == 0 || r < EJ_SCAN_ROUNDS) && more; r++) {
    int4 q[N];
#pragma unroll
    for (int j = 0; j < N; j++)
      if (more & (1u << j)) q[j] = __ldg(rv4 + sl[j] / 4);
#pragma unroll
    for (int j = 0; j < N; j++) {
      if (!(more & (1u << j))) continue;
      const int y[4] = {q[j].x, q[j].y, q[j].z, q[j].w};
      bool ended = false;
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const uint32_t idx = sl[j] + (uint32_t)e;
        if (idx >= s1[j] || ended) continue;
        if (y[e] == v[j]) {
          if (c[j] == 0) lo[j] = idx;
          c[j]++;
        } else if (c[j]) {
          ended = true;
        }
      }
      sl[j] += 4;
      if (ended || sl[j] >= s1[j]) more &= ~(1u << j);
    }
  }
  if (KIND != 0 && more) {
    upper = lower = 0;
#pragma unroll
    for (int j = 0; j < N; j++)
      if (more & (1u << j)) {
        if (c[j]) upper |= 1u << j; else lower |= 1u << j;
      }
    // a run's end: the first row past the run's key
    ej_search_rows<KIND, N>(rv, upper, true, key, sl, sh);
#pragma unroll
    for (int j = 0; j < N; j++)
      if (upper & (1u << j)) c[j] = sl[j] - lo[j];
    // no match yet: the first row at or past the key, and when it is the
    // value's, the run from there
    uint32_t found = 0;
    ej_search_rows<KIND, N>(rv, lower, false, key, sl, sh);
#pragma unroll
    for (int j = 0; j < N; j++)
      if ((lower & (1u << j)) && sl[j] < s1[j] && __ldg(rv + sl[j]) == v[j]) {
        lo[j] = sl[j];
        c[j] = 1;
        sl[j] += 1;
        sh[j] = s1[j];
        if (sl[j] < sh[j]) found |= 1u << j;  // a search needs a non-empty range
      }
    ej_search_rows<KIND, N>(rv, found, true, key, sl, sh);
#pragma unroll
    for (int j = 0; j < N; j++)
      if (found & (1u << j)) c[j] = sl[j] - lo[j];
  }
#pragma unroll
  for (int j = 0; j < N; j++) lo[j] -= t.voff;
}

// The key directory's slots of N probe hashes (dir.cuh): every probe loads
// the aligned 16-byte pair at its even home slot (hv >> shift) & ~1, then the
// next pair while both slots hold smaller hashes (slots are in hash order, so
// the second is the larger); the N walks advance together, one pair per
// round, so that a warp waits for as many dependent loads as its longest
// walk.  Out: a[j] the entry of the first slot whose hash is hv[j] or more,
// slot[j] that slot; when hasb[j], b[j] is the entry of the slot after it
// (else it is left to the caller to load).  ok[j] false: a[j].x = 0xFFFFFFFF.
template <int N>
__device__ __forceinline__ void ej_dir_walk(const uint2* __restrict__ dir, uint32_t shift, const uint32_t (&hv)[N],
                                            const bool (&ok)[N], uint2 (&a)[N], uint2 (&b)[N], bool (&hasb)[N],
                                            uint32_t (&slot)[N]) {
  const uint4* d4 = reinterpret_cast<const uint4*>(dir);  // 16-byte aligned
  uint4 q[N];
#pragma unroll
  for (int j = 0; j < N; j++) {
    slot[j] = (hv[j] >> shift) & ~1u;
    q[j] = make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
    if (ok[j]) q[j] = __ldg(d4 + (slot[j] >> 1));
  }
  uint32_t walk = 0;
#pragma unroll
  for (int j = 0; j < N; j++)
    if (q[j].z < hv[j]) walk |= 1u << j;
  while (walk) {  // the sentinels after the last entry end every walk
#pragma unroll
    for (int j = 0; j < N; j++)
      if (walk & (1u << j)) {
        slot[j] += 2;
        q[j] = __ldg(d4 + (slot[j] >> 1));
      }
#pragma unroll
    for (int j = 0; j < N; j++)
      if ((walk & (1u << j)) && q[j].z >= hv[j]) walk &= ~(1u << j);
  }
#pragma unroll
  for (int j = 0; j < N; j++) {
    hasb[j] = q[j].x >= hv[j];
    if (hasb[j]) {
      a[j] = make_uint2(q[j].x, q[j].y);
      b[j] = make_uint2(q[j].z, q[j].w);
    } else {
      a[j] = make_uint2(q[j].z, q[j].w);
      b[j] = a[j];
      slot[j] += 1;
    }
  }
}

// Runs of N probe values of a hash table at once: through the key directory
// (single tables that carry one), else through bucket bounds.  ok[j] false:
// c[j] = 0.
template <int N>
__device__ __forceinline__ void ej_find_runs_hash(const ej_table_view& t, const int32_t (&v)[N], const bool (&ok)[N],
                                                  uint32_t (&lo)[N], uint32_t (&c)[N]) {
  // a directory table whose build chose bucket bounds has bits = 0
  const uint32_t bits = t.dir ? __ldg(t.dir_bits) : 0u;
  if (bits) {
    // key directory: every slot holds the first key at or after it; a present
    // key's walk stops at its own slot, and the slot after it starts the next
    // run (the loops that look further are guards)
    uint32_t hv[N], slot[N];
    uint2 a[N], b[N];
    bool hasb[N];
#pragma unroll
    for (int j = 0; j < N; j++) hv[j] = ej_hash32((uint32_t)v[j]);
    ej_dir_walk<N>(t.dir, 32u - bits, hv, ok, a, b, hasb, slot);
    if (t.dir_packed) {
      // packed entries {hash, start << 5 | run length}: the length is in
      // hand unless the run has 31 rows or more (its end: the next start)
#pragma unroll
      for (int j = 0; j < N; j++) {
        lo[j] = 0u;
        c[j] = 0u;
        const uint32_t start = a[j].y >> 5;
        if (!ok[j] || a[j].x != hv[j] || start >= t.nR) continue;
        lo[j] = start;
        c[j] = a[j].y & 31u;
        if (c[j] == 31u) {
          uint32_t next = (hasb[j] ? b[j] : __ldg(t.dir + slot[j] + 1)).y >> 5;
          while (next == start) next = __ldg(t.dir + ++slot[j] + 1).y >> 5;
          c[j] = next - start;
        }
      }
    } else {
      // {hash, start}: the run ends at the next slot's start
#pragma unroll
      for (int j = 0; j < N; j++) {
        lo[j] = 0u;
        c[j] = 0u;
        if (!ok[j] || a[j].x != hv[j] || a[j].y >= t.nR) continue;
        uint2 nb = hasb[j] ? b[j] : __ldg(t.dir + slot[j] + 1);
        while (nb.y == a[j].y) nb = __ldg(t.dir + ++slot[j] + 1);
        lo[j] = a[j].y;
        c[j] = nb.y - a[j].y;
      }
    }
    return;
  }
  ej_find_runs_bucket<0, N>(t, v, ok, lo, c);
}

// runs of N probe values (ok[j] false: c[j] = 0)
template <int KIND, int N>
__device__ __forceinline__ void ej_find_runs(const ej_table_view& t, const int32_t (&v)[N], const bool (&ok)[N],
                                             uint32_t (&lo)[N], uint32_t (&c)[N]) {
  if (KIND == EJ_TABLE_HASH)
    ej_find_runs_hash<N>(t, v, ok, lo, c);
  else
    ej_find_runs_bucket<EJ_TABLE_SORTED, N>(t, v, ok, lo, c);
}
