// probe.cuh - where a probe value's matches lie in a table (device code).
//
// A table stores R as rkey[]/rval[] in one order (ej_table_view).  In both
// kinds the matches of a value v form one contiguous run [lo, lo + c):
//   EJ_TABLE_HASH    rows sorted by hash32(val); the run lies inside bucket
//                    b = top hb hash bits, [start[b], start[b+1]), found by
//                    scanning the bucket with 16-byte vector loads of rval;
//   EJ_TABLE_SORTED  rows sorted by val; lower and upper bounds by binary
//                    search, first over the fence (every 256th val), then
//                    inside one 256-row segment.
#pragma once

#include "ej_device.cuh"

__device__ __forceinline__ uint32_t ej_bucket_of(int32_t val, uint32_t hb) {
  return ej_hash32((uint32_t)val) >> (32u - hb);
}

template <int KIND>
struct EjRun;

template <>
struct EjRun<EJ_TABLE_HASH> {
  static __device__ __forceinline__ void find(const ej_table_view& t, int32_t v, uint32_t& lo, uint32_t& c) {
    const uint32_t b = ej_bucket_of(v, t.hb);
    const uint32_t s0 = __ldg(t.start + b), s1 = __ldg(t.start + b + 1);
    lo = s1;
    c = 0;
    bool ended = false;
    for (uint32_t i = s0 & ~3u; i < s1 && !ended; i += 4) {
      const int4 q = __ldg(reinterpret_cast<const int4*>(t.rval + i));
      const int x[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const uint32_t idx = i + (uint32_t)e;
        if (idx < s0 || idx >= s1) continue;
        if (x[e] == v) {
          if (c == 0) lo = idx;
          c++;
        } else if (c) {
          ended = true;  // rows are hash-sorted: the run of v is over
        }
      }
    }
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
