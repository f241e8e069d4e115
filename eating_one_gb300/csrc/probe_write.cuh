// probe_write.cuh - count and write passes of the probe (device code), shared
// by the single-join kernels (hash_join.cu) and the batched ones (batch.cu).
//
// The unit of work is a warp tile of 128 probes: lane l holds probes 32j + l
// (j = 0..3), so every load of the probe tuples is coalesced and the warp's
// output rows form one contiguous range.  Three launches, no inter-warp
// waiting anywhere:
//   count  finds the runs of the four probes (loads issued together,
//          probe.cuh), stores each probe's run descriptor (lo, length) and
//          the warp tile's row total;
//   scan   of the warp-tile totals: every warp tile's output offset;
//   write  reads the probes and their descriptors (both coalesced), fetches
//          the keys of each run's first PW_PREFETCH rows (one round of loads),
//          and writes the rows group by group (32 probes): each lane places
//          its rows in the warp's 4 KB shared-memory buffer (slots XOR-
//          swizzled, so that lanes whose runs have equal lengths do not
//          collide on the banks) and the warp copies the buffer out with
//          coalesced 16-byte streaming stores when the next group does not
//          fit; a group with more rows than the buffer goes 32 consecutive
//          rows per round, lane i finding the probe of row i with a five-step
//          shuffle search over the lanes' row prefixes.
// The *_count entry points run the count pass without descriptors.
#pragma once

#include "ej_device.cuh"
#include "probe.cuh"

constexpr int PR_THREADS = 256;
constexpr int PR_WARPS = PR_THREADS / 32;
constexpr int PR_ITEMS = 4;
constexpr int PR_WTILE = 32 * PR_ITEMS;         // 128 probes per warp tile
constexpr int PR_TILE = PR_THREADS * PR_ITEMS;  // 1024 probes per block
constexpr int PW_PREFETCH = 4;                  // run keys held in registers per probe
constexpr uint32_t PW_STAGE_ROWS = 256;         // staged rows per warp (4 KB)
constexpr uint32_t PW_BIG_RUN = 1u << 26;       // a run at least this long makes its group use 64-bit prefixes
constexpr uint32_t NULL_RUN = 0xFFFFFFFFu;      // OUTER: the NULL-extended row

struct EjProbeWarp {
  int2 s[PR_ITEMS];
  uint32_t lo[PR_ITEMS], cnt[PR_ITEMS];
};

// slot of staged row r: rows r and r + 8k land on different 16-byte bank
// groups for k = 1..7
__device__ __forceinline__ uint32_t ej_stage_slot(uint32_t r) { return r ^ ((r >> 3) & 7u); }

// probes [base, min(base + 128, nP)): tuples and runs (OUTER: an unmatched
// probe gets one row, marked by lo = NULL_RUN)
template <int KIND, bool OUTER>
__device__ __forceinline__ void ej_probe_runs_warp(const ej_tuple* __restrict__ P, uint64_t base, uint64_t nP,
                                                   const ej_table_view& t, EjProbeWarp& w) {
  const unsigned int lane = threadIdx.x & 31u;
  int32_t v[PR_ITEMS];
  bool ok[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * 32 + lane;
    ok[j] = idx < nP;
    w.s[j] = ok[j] ? __ldcs(reinterpret_cast<const int2*>(P) + idx) : make_int2(0, 0);
    v[j] = w.s[j].y;
  }
  ej_find_runs<KIND, PR_ITEMS>(t, v, ok, w.lo, w.cnt);
  if (OUTER) {
#pragma unroll
    for (int j = 0; j < PR_ITEMS; j++)
      if (ok[j] && w.cnt[j] == 0) {
        w.cnt[j] = 1;
        w.lo[j] = NULL_RUN;
      }
  }
}

// rows of a warp tile (every lane returns the total)
template <int KIND, bool OUTER>
__device__ __forceinline__ unsigned long long ej_probe_count_warp(const ej_tuple* __restrict__ P, uint64_t base,
                                                                  uint64_t nP, const ej_table_view& t) {
  EjProbeWarp w;
  ej_probe_runs_warp<KIND, OUTER>(P, base, nP, t, w);
  unsigned long long mine = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) mine += w.cnt[j];
  return ej_warp_sum<unsigned long long>(mine);
}

// rows of group j of 32 probes; incl: the lane's inclusive 32-bit prefix when
// no run of the group is PW_BIG_RUN long (big = false), else unused
__device__ __forceinline__ unsigned long long ej_group_rows(uint32_t c, uint32_t& incl, bool& big) {
  big = __any_sync(EJ_FULL_MASK, c >= PW_BIG_RUN);
  if (big) return ej_warp_sum<unsigned long long>(c);
  incl = ej_warp_inclusive_sum<uint32_t>(c);
  return __shfl_sync(EJ_FULL_MASK, incl, 31);
}

// keys of the first PW_PREFETCH rows of every run (rkey - voff is 16-byte
// aligned and the column is padded, so every load stays inside it), in one
// of two schemes fixed at compile time (the L1 data path pays for the bytes
// it delivers; both schemes in one kernel cost more than either saves):
//   EJ_KEYS_WINDOW  the aligned 8-key window holding the first four keys, one
//                   or two 16-byte loads (single tables: C3's runs of four);
//   EJ_KEYS_CHUNKS  the aligned 8-byte chunks holding them, one to three
//                   loads (batched tables, whose runs are mostly of one or
//                   two rows).
enum { EJ_KEYS_WINDOW = 0, EJ_KEYS_CHUNKS = 1 };
template <int KEYS = EJ_KEYS_WINDOW>
__device__ __forceinline__ void ej_probe_prefetch(const ej_table_view& t, const EjProbeWarp& w,
                                                  int32_t (&kk)[PR_ITEMS][PW_PREFETCH]) {
  static_assert(PW_PREFETCH == 4, "the window holds 4 keys past any offset");
  constexpr bool chunks = KEYS == EJ_KEYS_CHUNKS;
  const int4* rk4 = reinterpret_cast<const int4*>(t.rkey - t.voff);
  const int2* rk2 = reinterpret_cast<const int2*>(t.rkey - t.voff);
  int4 qa[PR_ITEMS], qb[PR_ITEMS];
  uint32_t o[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    qa[j] = qb[j] = make_int4(EJ_NULL_KEY, EJ_NULL_KEY, EJ_NULL_KEY, EJ_NULL_KEY);
    o[j] = 0;
    if (w.lo[j] != NULL_RUN && w.cnt[j]) {
      const uint32_t p = w.lo[j] + t.voff;
      if (chunks) {  // keys p .. p + min(cnt, 4) - 1 from the 8-byte chunks holding them
        const uint32_t last = (p + min(w.cnt[j], (uint32_t)PW_PREFETCH) - 1u) / 2u;
        o[j] = p & 1u;
        const int2 a = __ldg(rk2 + p / 2);
        int2 b = make_int2(EJ_NULL_KEY, EJ_NULL_KEY), c = b;
        if (last >= p / 2 + 1u) b = __ldg(rk2 + p / 2 + 1);
        if (last >= p / 2 + 2u) c = __ldg(rk2 + p / 2 + 2);
        qa[j] = make_int4(a.x, a.y, b.x, b.y);
        qb[j].x = c.x;
        qb[j].y = c.y;
      } else {
        o[j] = p & 3u;
        qa[j] = __ldg(rk4 + p / 4);
        if (o[j] + min(w.cnt[j], (uint32_t)PW_PREFETCH) > 4u) qb[j] = __ldg(rk4 + p / 4 + 1);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const int32_t x[8] = {qa[j].x, qa[j].y, qa[j].z, qa[j].w, qb[j].x, qb[j].y, qb[j].z, qb[j].w};
#pragma unroll
    for (int e = 0; e < PW_PREFETCH; e++) {
      // x[o + e] with static indices only
      const int32_t v = o[j] == 0 ? x[e] : o[j] == 1 ? x[e + 1] : o[j] == 2 ? x[e + 2] : x[e + 3];
      kk[j][e] = (uint32_t)e < w.cnt[j] ? v : EJ_NULL_KEY;
    }
  }
}

// group rows of one lane: buffer rows [r, r + c), keys from kk for the first
// PW_PREFETCH (PREFETCHED) and from the table for the rest
template <bool PREFETCHED>
__device__ __forceinline__ void ej_stage_rows(int4* stage, uint32_t r, uint32_t c, const int32_t (&kk)[PW_PREFETCH],
                                              uint32_t lo, int32_t sk, int32_t sv, const ej_table_view& t) {
  const int32_t rv = lo == NULL_RUN ? EJ_NULL_KEY : sv;
  uint32_t e = 0;
  if (PREFETCHED) {
#pragma unroll
    for (int q = 0; q < PW_PREFETCH; q++)
      if ((uint32_t)q < c) stage[ej_stage_slot(r + q)] = make_int4(kk[q], rv, sk, sv);
    e = PW_PREFETCH;
  }
  // OUTER: a NULL-extended row (lo = NULL_RUN, c = 1) has no table row to read
  for (; e < c; e++)
    stage[ej_stage_slot(r + e)] = make_int4(lo == NULL_RUN ? EJ_NULL_KEY : __ldg(t.rkey + lo + e), rv, sk, sv);
}

// buffer rows [0, n) to out[a, a + n) (rows at or past cap dropped)
__device__ __forceinline__ void ej_flush_stage(const int4* stage, uint32_t n, unsigned long long a,
                                               ej_result* __restrict__ out, uint64_t cap) {
  const unsigned int lane = threadIdx.x & 31u;
  __syncwarp();
  for (uint32_t r = lane; r < n; r += 32)
    if (a + r < cap) __stcs(reinterpret_cast<int4*>(out + a + r), stage[ej_stage_slot(r)]);
  __syncwarp();
}

// a group with more rows than the buffer: 32 consecutive rows per round from out[a]
__device__ __forceinline__ void ej_emit_big_group(uint32_t c, unsigned long long gsum, uint32_t lo, int32_t sk,
                                                  int32_t sv, const ej_table_view& t, unsigned long long a,
                                                  ej_result* __restrict__ out, uint64_t cap) {
  const unsigned int lane = threadIdx.x & 31u;
  const unsigned long long pincl = ej_warp_inclusive_sum<unsigned long long>(c);
  const unsigned long long pre = pincl - c;  // group-relative first row of this lane
  for (unsigned long long o0 = 0; o0 < gsum && a + o0 < cap; o0 += 32) {
    const unsigned long long o = o0 + lane;
    int src = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const unsigned long long x = __shfl_sync(EJ_FULL_MASK, pre, src + step);
      if (x <= o) src += step;
    }
    const uint32_t e = (uint32_t)(o - __shfl_sync(EJ_FULL_MASK, pre, src));
    const uint32_t rlo = __shfl_sync(EJ_FULL_MASK, lo, src);
    const int32_t rk = __shfl_sync(EJ_FULL_MASK, sk, src);
    const int32_t rs = __shfl_sync(EJ_FULL_MASK, sv, src);
    if (o < gsum && a + o < cap) {
      const int32_t key = rlo == NULL_RUN ? EJ_NULL_KEY : __ldg(t.rkey + rlo + e);
      __stcs(reinterpret_cast<int4*>(out + a + o), make_int4(key, rlo == NULL_RUN ? EJ_NULL_KEY : rs, rk, rs));
    }
  }
}

// The rows of a warp tile from out[off] on (rows at or past cap dropped):
// group by group through the warp's buffer; kk: the prefetched keys of the
// first rows of every run.
__device__ __forceinline__ void ej_emit_warp(const EjProbeWarp& w, const int32_t (&kk)[PR_ITEMS][PW_PREFETCH],
                                             const ej_table_view& t, unsigned long long a,
                                             ej_result* __restrict__ out, uint64_t cap, int4* stage) {
  // runs of at most one row throughout the tile (unique keys; an outer
  // join's NULL-extended rows): each group's rows go straight out in lane
  // order, positions from one ballot, no staging and no scans
  bool one = true;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) one &= w.cnt[j] <= 1u;
  if (__all_sync(EJ_FULL_MASK, one)) {
    const unsigned int lt = ej_lanemask_lt();
#pragma unroll
    for (int j = 0; j < PR_ITEMS; j++) {
      const unsigned int b = __ballot_sync(EJ_FULL_MASK, w.cnt[j] != 0u);
      const unsigned long long p = a + (unsigned)__popc(b & lt);
      if (w.cnt[j] && p < cap)
        __stcs(reinterpret_cast<int4*>(out + p),
               make_int4(kk[j][0], w.lo[j] == NULL_RUN ? EJ_NULL_KEY : w.s[j].y, w.s[j].x, w.s[j].y));
      a += (unsigned)__popc(b);
    }
    return;
  }
  uint32_t fill = 0;  // staged rows, the first of them at out[a]
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    uint32_t incl = 0;
    bool big;
    const unsigned long long gsum = ej_group_rows(w.cnt[j], incl, big);
    if (gsum == 0) continue;
    if (!big && gsum <= PW_STAGE_ROWS) {
      if (gsum > PW_STAGE_ROWS - fill) {
        ej_flush_stage(stage, fill, a, out, cap);
        a += fill;
        fill = 0;
      }
      ej_stage_rows<true>(stage, fill + incl - w.cnt[j], w.cnt[j], kk[j], w.lo[j], w.s[j].x, w.s[j].y, t);
      fill += (uint32_t)gsum;
    } else {
      ej_flush_stage(stage, fill, a, out, cap);
      a += fill;
      fill = 0;
      if (a < cap) ej_emit_big_group(w.cnt[j], gsum, w.lo[j], w.s[j].x, w.s[j].y, t, a, out, cap);
      a += gsum;
    }
  }
  if (fill) ej_flush_stage(stage, fill, a, out, cap);
}

// Run descriptors stored by the count pass for the write pass, in one of two
// forms: EJ_DESC_WIDE, 8 bytes (lo, length); EJ_DESC_PACKED, 4 bytes
// (lo << 5 | length) for tables of fewer than 2^27 rows, with the length
// field EJ_PACKED_ESCAPE meaning "31 rows or more, or a NULL-extended row:
// find the run again" (the write pass then repeats the find for its tile).
enum { EJ_DESC_NONE = 0, EJ_DESC_WIDE = 1, EJ_DESC_PACKED = 2 };
constexpr uint64_t EJ_PACKED_MAX_ROWS = 1ull << 27;
constexpr uint32_t EJ_PACKED_ESCAPE = 31;

__device__ __forceinline__ uint32_t ej_pack_run(uint32_t lo, uint32_t cnt) {
  if (cnt == 0) return 0u;
  if (cnt >= EJ_PACKED_ESCAPE || lo == NULL_RUN) return EJ_PACKED_ESCAPE;
  return (lo << 5) | cnt;
}

// count pass of a warp tile; DESC: also stores each probe's run (lo, length)
// in desc[probe] (OUTER: (NULL_RUN, 1) for a probe without matches), wide or
// packed.  Every lane returns the warp tile's rows.
template <int KIND, bool OUTER, int DESC>
__device__ __forceinline__ unsigned long long ej_probe_count_warp_desc(const ej_tuple* __restrict__ P, uint64_t base,
                                                                       uint64_t nP, const ej_table_view& t,
                                                                       void* __restrict__ desc) {
  const unsigned int lane = threadIdx.x & 31u;
  EjProbeWarp w;
  ej_probe_runs_warp<KIND, OUTER>(P, base, nP, t, w);
  unsigned long long mine = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    mine += w.cnt[j];
    const uint64_t idx = base + (uint64_t)j * 32 + lane;
    if (DESC == EJ_DESC_WIDE && idx < nP) __stcs(static_cast<uint2*>(desc) + idx, make_uint2(w.lo[j], w.cnt[j]));
    if (DESC == EJ_DESC_PACKED && idx < nP)
      __stcs(static_cast<unsigned int*>(desc) + idx, ej_pack_run(w.lo[j], w.cnt[j]));
  }
  return ej_warp_sum<unsigned long long>(mine);
}

// write pass of a warp tile whose output starts at out[off], from the
// descriptors of the count pass (DESC: their form; a packed escape makes the
// warp find its tile's runs again, KIND and OUTER as in the count pass)
template <int KIND, bool OUTER, int DESC>
__device__ __forceinline__ void ej_probe_write_warp(const ej_tuple* __restrict__ P, const void* __restrict__ desc,
                                                    uint64_t base, uint64_t nP, const ej_table_view& t,
                                                    unsigned long long off, ej_result* __restrict__ out,
                                                    uint64_t cap, int4* stage) {
  const unsigned int lane = threadIdx.x & 31u;
  EjProbeWarp w;
  bool escape = false;
#pragma unroll
  for (int j = 0; j < PR_ITEMS && DESC != EJ_DESC_NONE; j++) {
    const uint64_t idx = base + (uint64_t)j * 32 + lane;
    const bool ok = idx < nP;
    w.s[j] = ok ? __ldcs(reinterpret_cast<const int2*>(P) + idx) : make_int2(0, 0);
    if (DESC == EJ_DESC_PACKED) {
      const uint32_t d = ok ? __ldcs(static_cast<const unsigned int*>(desc) + idx) : 0u;
      w.lo[j] = d >> 5;
      w.cnt[j] = d & 31u;
      escape |= w.cnt[j] == EJ_PACKED_ESCAPE;
    } else {
      const uint2 d = ok ? __ldcs(static_cast<const uint2*>(desc) + idx) : make_uint2(0u, 0u);
      w.lo[j] = d.x;
      w.cnt[j] = d.y;
    }
  }
  // no descriptors (a packed key directory answers a probe in one load): the
  // count pass's find, repeated
  if (DESC == EJ_DESC_NONE || (DESC == EJ_DESC_PACKED && __any_sync(EJ_FULL_MASK, escape)))
    ej_probe_runs_warp<KIND, OUTER>(P, base, nP, t, w);
  int32_t kk[PR_ITEMS][PW_PREFETCH];
  ej_probe_prefetch(t, w, kk);
  ej_emit_warp(w, kk, t, off, out, cap, stage);
}
