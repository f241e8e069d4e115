// probe_write.cuh - count and write passes of the probe (device code), shared
// by the single-join kernels (hash_join.cu) and the batched ones (batch.cu).
//
// A tile of 1024 probes is eight warp tiles of 128: lane l of warp w holds
// probes 128w + 32j + l (j = 0..3), so every load of the probe tuples is
// coalesced and the warp's output rows form one contiguous range.  The write
// pass does one walk over the table per probe:
//   1. find the runs of the four probes (loads issued together, probe.cuh)
//      and fetch the keys of each run's first PW_PREFETCH rows;
//   2. warp totals, one block barrier, and the tile's output offset from the
//      preceding tiles of its chain by decoupled look-back (warp 0);
//   3. a warp tile with at most PW_STAGE_ROWS rows (every tile of a join
//      with up to four matches per probe) stages all of them in the warp's
//      8 KB shared-memory buffer while warp 0 looks back, each lane placing
//      its own rows (slots XOR-swizzled, so that lanes whose runs have equal
//      lengths do not collide on the banks); after the second block barrier
//      the warp copies the buffer out with coalesced 16-byte streaming stores;
//   4. larger warp tiles go group by group (32 probes) once the offset is
//      known, through the same buffer, and a group with more rows than the
//      buffer 32 consecutive rows per round, lane i finding the probe of row
//      i with a five-step shuffle search over the lanes' row prefixes.
// The count pass (the *_count entry points) stores the totals of warp tiles.
#pragma once

#include "ej_device.cuh"
#include "probe.cuh"

constexpr int PR_THREADS = 256;
constexpr int PR_WARPS = PR_THREADS / 32;
constexpr int PR_ITEMS = 4;
constexpr int PR_WTILE = 32 * PR_ITEMS;         // 128 probes per warp tile
constexpr int PR_TILE = PR_THREADS * PR_ITEMS;  // 1024 probes per block
constexpr int PW_PREFETCH = 4;                  // run keys held in registers per probe
constexpr uint32_t PW_STAGE_ROWS = 512;         // staged rows per warp (8 KB): four rows per probe
constexpr uint32_t PW_BIG_RUN = 1u << 26;       // a run at least this long makes its group use 64-bit prefixes
constexpr uint32_t NULL_RUN = 0xFFFFFFFFu;      // OUTER: the NULL-extended row

struct EjProbeWarp {
  int2 s[PR_ITEMS];
  uint32_t lo[PR_ITEMS], cnt[PR_ITEMS];
};

// dynamic shared memory of a write block (64 KB staging)
struct PwSmem {
  int4 stage[PR_WARPS][PW_STAGE_ROWS];
  unsigned long long wtot[PR_WARPS];  // rows of each warp
  unsigned long long woff[PR_WARPS];  // output offset of each warp within the tile
  unsigned long long tile_off;
  unsigned int tile;
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

// keys of the first PW_PREFETCH rows of every run
__device__ __forceinline__ void ej_probe_prefetch(const ej_table_view& t, const EjProbeWarp& w,
                                                  int32_t (&kk)[PR_ITEMS][PW_PREFETCH]) {
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++)
#pragma unroll
    for (int e = 0; e < PW_PREFETCH; e++)
      kk[j][e] = (w.lo[j] != NULL_RUN && (uint32_t)e < w.cnt[j]) ? __ldg(t.rkey + w.lo[j] + e) : EJ_NULL_KEY;
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

// Stage every row of a warp tile with at most PW_STAGE_ROWS rows (no output
// offset needed yet): the keys of the first rows of every run are loaded
// together, then each lane places its rows.
__device__ __forceinline__ void ej_stage_warp(const EjProbeWarp& w, const ej_table_view& t, int4* stage) {
  int32_t kk[PR_ITEMS][PW_PREFETCH];
  ej_probe_prefetch(t, w, kk);
  uint32_t gbase = 0;  // buffer row of the group's first row
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint32_t incl = ej_warp_inclusive_sum<uint32_t>(w.cnt[j]);  // the warp has at most 512 rows
    ej_stage_rows<true>(stage, gbase + incl - w.cnt[j], w.cnt[j], kk[j], w.lo[j], w.s[j].x, w.s[j].y, t);
    gbase += __shfl_sync(EJ_FULL_MASK, incl, 31);
  }
}

// A warp tile with more rows than the buffer, from out[a] on (rows at or past
// cap dropped): group by group through the buffer.
__device__ __forceinline__ void ej_emit_warp_groups(const EjProbeWarp& w, const ej_table_view& t,
                                                    unsigned long long a, ej_result* __restrict__ out, uint64_t cap,
                                                    int4* stage) {
  const int32_t none[PW_PREFETCH] = {};
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
      ej_stage_rows<false>(stage, fill + incl - w.cnt[j], w.cnt[j], none, w.lo[j], w.s[j].x, w.s[j].y, t);
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

// One tile: probes [base, min(base + 1024, nP)) of P against table t; `tile`
// is the tile's index in its look-back chain (lb_status), `last` marks the
// chain's last tile, which stores the chain's total in *d_total.  The caller
// has claimed the tile and synchronised the block.
template <int KIND, bool OUTER>
__device__ __forceinline__ void ej_probe_write_tile(PwSmem& sm, const ej_tuple* __restrict__ P, uint64_t base,
                                                    uint64_t nP, const ej_table_view& t,
                                                    unsigned long long* lb_status, uint64_t tile, bool last,
                                                    ej_result* __restrict__ out, uint64_t cap,
                                                    unsigned long long* d_total, ej_dev_status* st) {
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // 1. runs
  EjProbeWarp w;
  ej_probe_runs_warp<KIND, OUTER>(P, base + (uint64_t)warp * PR_WTILE, nP, t, w);

  // 2. warp totals; warp 0 publishes the tile's total, every warp whose rows
  //    fit stages them, then warp 0 resolves the tile's offset
  unsigned long long mine = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) mine += w.cnt[j];
  const unsigned long long wrun = ej_warp_sum<unsigned long long>(mine);
  if (lane == 0) sm.wtot[warp] = wrun;
  __syncthreads();
  unsigned long long total = 0;
  if (warp == 0) {
    const unsigned long long x = lane < PR_WARPS ? sm.wtot[lane] : 0ull;
    const unsigned long long incl = ej_warp_inclusive_sum<unsigned long long>(x);
    if (lane < PR_WARPS) sm.woff[lane] = incl - x;
    total = __shfl_sync(EJ_FULL_MASK, incl, 31);
    ej_lookback_publish(lb_status, tile, total);
  }
  const bool fits = wrun <= PW_STAGE_ROWS;
  if (fits && wrun) ej_stage_warp(w, t, sm.stage[warp]);
  if (warp == 0) {
    const unsigned long long off = ej_lookback_resolve(lb_status, tile, total, st, 3u);
    if (lane == 0) {
      sm.tile_off = off;
      if (last) {
        *d_total = off + total;
        if (off + total > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
      }
    }
  }
  __syncthreads();
  const unsigned long long gbase = sm.tile_off + sm.woff[warp];
  if (gbase >= cap || wrun == 0) return;

  // 3./4. rows of this warp
  if (fits)
    ej_flush_stage(sm.stage[warp], (uint32_t)wrun, gbase, out, cap);
  else
    ej_emit_warp_groups(w, t, gbase, out, cap, sm.stage[warp]);
}
