// probe.cuh - where a probe value's matches lie in a table (device code).
//
// A table stores R as rkey[]/rval[] in one order (ej_table_view).  In both
// kinds the matches of a value v form one contiguous run [lo, lo + c):
//   EJ_TABLE_HASH    rows sorted by hash32(val).  Single tables carry a key
//                    directory (8-byte entries {hash, lo} in hash order,
//                    linear probing from slot hash >> (32 - bits), each slot
//                    holding the first key at or after it, so c is the next
//                    slot's start minus lo); batched tables carry bucket bounds: the run
//                    lies inside bucket b = top hb hash bits, rows
//                    [bucket[b].x, bucket[b].y) (one 8-byte load), found by
//                    scanning the bucket with 16-byte vector loads of rval;
//   EJ_TABLE_SORTED  rows sorted by val; lower and upper bounds by binary
//                    search, first over the fence (every 256th val), then
//                    inside one 256-row segment.
#pragma once

#include "ej_device.cuh"

__device__ __forceinline__ uint32_t ej_bucket_of(int32_t val, uint32_t hb) {
  return ej_hash32((uint32_t)val) >> (32u - hb);
}

// Table build: bucket b begins at row i, so bucket[b].x = i (b < nb) and the
// previous bucket ends there, bucket[b - 1].y = i (b > 0).
__device__ __forceinline__ void ej_set_bucket_begin(uint2* bucket, int64_t b, int64_t nb, uint32_t i) {
  uint32_t* w = reinterpret_cast<uint32_t*>(bucket);
  if (b < nb) w[2 * b] = i;
  if (b > 0) w[2 * b - 1] = i;
}

// Table build, one warp: the bounds of the buckets that begin at rows
// [r0, r0 + 256) of a hash-sorted column of n rows; row n (when in range) is
// the end, which begins the buckets past the last row's.  Lane l looks at
// rows r0 + 32k + l (coalesced loads, all issued together) and takes the
// bucket of the row before from its neighbour lane.
__device__ __forceinline__ void ej_bucket_bounds_warp(const int32_t* __restrict__ rval, uint64_t n, uint64_t r0,
                                                      uint32_t hb, uint2* __restrict__ bucket) {
  const unsigned int lane = threadIdx.x & 31u;
  const int32_t nb = (int32_t)(1u << hb);
  int32_t cur[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint64_t i = r0 + (uint64_t)k * 32 + lane;
    cur[k] = i < n ? (int32_t)ej_bucket_of(rval[i], hb) : nb;
  }
  int32_t carry = -1;  // bucket of row r0 + 32k - 1
  if (r0 > 0) carry = r0 - 1 < n ? (int32_t)ej_bucket_of(rval[r0 - 1], hb) : nb;
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

template <int KIND>
struct EjRun;

// Runs of N probe values at once, in three rounds of independent loads (bucket
// bounds of every value, then the first 32 bytes of every bucket); only a
// bucket longer than that continues in a loop.  ok[j] false: c[j] = 0.
template <int N>
__device__ __forceinline__ void ej_find_runs_hash(const ej_table_view& t, const int32_t (&v)[N], const bool (&ok)[N],
                                                  uint32_t (&lo)[N], uint32_t (&c)[N]) {
  if (t.dir) {
    // key directory: every slot holds the first key at or after it; walk past
    // smaller hashes, then the run ends at the first slot with another start
    // (slot + 1 never passes the sentinels after the last entry)
    const uint32_t shift = 32u - __ldg(t.dir_bits);
    uint32_t hv[N], slot[N];
    uint2 a[N], b[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
      hv[j] = ej_hash32((uint32_t)v[j]);
      slot[j] = hv[j] >> shift;
      a[j] = b[j] = make_uint2(0u, 0u);
      if (ok[j]) {
        // the 16-byte aligned slot pair holding the home slot (the directory
        // starts 16-byte aligned): both slots needed when it is even
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(t.dir) + (slot[j] >> 1));
        if (slot[j] & 1u) {
          a[j] = make_uint2(q.z, q.w);
          b[j] = __ldg(t.dir + slot[j] + 1);
        } else {
          a[j] = make_uint2(q.x, q.y);
          b[j] = make_uint2(q.z, q.w);
        }
      }
    }
    // the N walks advance together, one slot per round, so that a warp waits
    // for as many dependent loads as its longest walk, not for their sum
    uint32_t walk = 0;
#pragma unroll
    for (int j = 0; j < N; j++)
      if (ok[j] && a[j].x < hv[j]) walk |= 1u << j;
    while (walk) {
#pragma unroll
      for (int j = 0; j < N; j++)
        if (walk & (1u << j)) {
          a[j] = b[j];
          b[j] = __ldg(t.dir + ++slot[j] + 1);
        }
#pragma unroll
      for (int j = 0; j < N; j++)
        if ((walk & (1u << j)) && a[j].x >= hv[j]) walk &= ~(1u << j);
    }
#pragma unroll
    for (int j = 0; j < N; j++) {
      lo[j] = 0u;
      c[j] = 0u;
      if (!ok[j] || a[j].x != hv[j] || a[j].y >= t.nR) continue;
      // a present key's home slot is never a gap, so the walk stops at the
      // key's own slot and the next slot starts another run; the loop is a guard
      while (b[j].y == a[j].y) b[j] = __ldg(t.dir + ++slot[j] + 1);
      lo[j] = a[j].y;
      c[j] = b[j].y - a[j].y;
    }
    return;
  }
  uint32_t s0[N], s1[N];
#pragma unroll
  for (int j = 0; j < N; j++) {
    s0[j] = s1[j] = 0;
    if (ok[j]) {
      const uint2 bb = __ldg(t.bucket + ej_bucket_of(v[j], t.hb));
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
  uint32_t more = 0;  // bit j: the run or the search of probe j goes on past the 8 loaded values
  uint32_t next[N];   // the next 4 values to scan
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
    // rows are hash-sorted, so the matches are one contiguous run
    c[j] = __popc(eq);
    lo[j] = c[j] ? base + (uint32_t)(__ffs(eq) - 1) : s1[j];
    // a run goes on past the 8 loaded values only if it reaches their end; with
    // no match yet, the search goes on only if the bucket does
    const bool ended = c[j] ? !(eq & 0x80u) : (to < 8u);
    next[j] = base + 8;
    if (!ended && next[j] < s1[j]) more |= 1u << j;
  }
  // the N scans advance together, 4 values per round, so that a warp waits
  // for as many dependent loads as its longest scan, not for their sum
  while (more) {
    int4 q[N];
#pragma unroll
    for (int j = 0; j < N; j++)
      if (more & (1u << j)) q[j] = __ldg(rv4 + next[j] / 4);
#pragma unroll
    for (int j = 0; j < N; j++) {
      if (!(more & (1u << j))) continue;
      const int y[4] = {q[j].x, q[j].y, q[j].z, q[j].w};
      bool ended = false;
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const uint32_t idx = next[j] + (uint32_t)e;
        if (idx >= s1[j] || ended) continue;
        if (y[e] == v[j]) {
          if (c[j] == 0) lo[j] = idx;
          c[j]++;
        } else if (c[j]) {
          ended = true;
        }
      }
      next[j] += 4;
      if (ended || next[j] >= s1[j]) more &= ~(1u << j);
    }
  }
#pragma unroll
  for (int j = 0; j < N; j++) lo[j] -= t.voff;
}

template <>
struct EjRun<EJ_TABLE_HASH> {
  static __device__ __forceinline__ void find(const ej_table_view& t, int32_t v, uint32_t& lo, uint32_t& c) {
    const int32_t vv[1] = {v};
    const bool ok[1] = {true};
    uint32_t l[1], n[1];
    ej_find_runs_hash<1>(t, vv, ok, l, n);
    lo = l[0];
    c = n[0];
  }
};

// first index in [lo, hi) whose val is >= v (STRICT: > v); hi when none
template <bool STRICT>
__device__ __forceinline__ uint32_t ej_sorted_bound(const int32_t* vals, uint32_t lo, uint32_t hi, int32_t v) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    const int32_t x = __ldg(vals + mid);
    if (STRICT ? (x <= v) : (x < v)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <bool STRICT>
__device__ __forceinline__ uint32_t ej_fenced_bound(const ej_table_view& t, int32_t v) {
  uint32_t f = ej_sorted_bound<STRICT>(t.fence, 0u, t.nfence, v);  // first fence entry >= v (> v)
  if (f == 0) return 0;
  const uint64_t seg_lo = (uint64_t)(f - 1) * EJ_FENCE_STRIDE;
  const uint64_t seg_hi = min((uint64_t)f * EJ_FENCE_STRIDE, t.nR);
  return ej_sorted_bound<STRICT>(t.rval, (uint32_t)seg_lo, (uint32_t)seg_hi, v);
}

template <>
struct EjRun<EJ_TABLE_SORTED> {
  static __device__ __forceinline__ void find(const ej_table_view& t, int32_t v, uint32_t& lo, uint32_t& c) {
    lo = ej_fenced_bound<false>(t, v);
    c = ej_fenced_bound<true>(t, v) - lo;
  }
};

// runs of N probe values (ok[j] false: c[j] = 0)
template <int KIND, int N>
__device__ __forceinline__ void ej_find_runs(const ej_table_view& t, const int32_t (&v)[N], const bool (&ok)[N],
                                             uint32_t (&lo)[N], uint32_t (&c)[N]) {
  if (KIND == EJ_TABLE_HASH) {
    ej_find_runs_hash<N>(t, v, ok, lo, c);
  } else {
#pragma unroll
    for (int j = 0; j < N; j++) {
      lo[j] = 0;
      c[j] = 0;
      if (ok[j]) EjRun<EJ_TABLE_SORTED>::find(t, v[j], lo[j], c[j]);
    }
  }
}
