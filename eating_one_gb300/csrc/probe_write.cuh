// probe_write.cuh - one tile of the write pass (device code), shared by the
// single-join write kernel (hash_join.cu) and the batched one (batch.cu).
//
// A tile of 1024 probes: warp w owns probes [128w, 128w + 128), lane l holds
// probes 32j + l (j = 0..3), so every load of the probe tuples is coalesced
// and the warp's output rows are one contiguous range.  Steps:
//   1. runs of all four probes (their loads issued together, probe.cuh); the
//      keys of the first PW_PREFETCH rows of every run go to registers;
//   2. warp scans of the run lengths, one block barrier to add up the warp
//      totals, and the tile's output offset from the preceding tiles of its
//      chain by decoupled look-back (warp 0);
//   3. each warp writes its own rows, 32 consecutive rows per round: lane i
//      finds the probe of row i with a five-step shuffle search over the
//      lanes' prefixes, takes the key from that lane's registers (or from the
//      table past the prefetched rows), and all lanes store 512 contiguous
//      bytes with 16-byte streaming stores.
// Probes with many matches simply take more rounds of their warp.
#pragma once

#include "ej_device.cuh"
#include "probe.cuh"

constexpr int PR_THREADS = 256;
constexpr int PR_WARPS = PR_THREADS / 32;
constexpr int PR_ITEMS = 4;
constexpr int PR_TILE = PR_THREADS * PR_ITEMS;  // 1024 probes
constexpr int PW_PREFETCH = 4;                  // run keys held in registers per probe
constexpr uint32_t NULL_RUN = 0xFFFFFFFFu;      // OUTER: the NULL-extended row

struct PwSmem {
  unsigned long long wtot[PR_WARPS];  // rows of each warp
  unsigned long long woff[PR_WARPS];  // output offset of each warp within the tile
  unsigned long long tile_off;
  unsigned long long total;
  unsigned int tile;
};

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
  const uint64_t wbase = base + (uint64_t)warp * (32 * PR_ITEMS);

  // 1. runs
  int2 s[PR_ITEMS];
  int32_t v[PR_ITEMS];
  bool ok[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = wbase + (uint64_t)j * 32 + lane;
    ok[j] = idx < nP;
    s[j] = ok[j] ? __ldcs(reinterpret_cast<const int2*>(P) + idx) : make_int2(0, 0);
    v[j] = s[j].y;
  }
  uint32_t lo[PR_ITEMS], cnt[PR_ITEMS];
  ej_find_runs<KIND, PR_ITEMS>(t, v, ok, lo, cnt);
  int32_t kk[PR_ITEMS][PW_PREFETCH];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    if (OUTER && ok[j] && cnt[j] == 0) {
      cnt[j] = 1;
      lo[j] = NULL_RUN;
    }
#pragma unroll
    for (int e = 0; e < PW_PREFETCH; e++)
      kk[j][e] = (lo[j] != NULL_RUN && (uint32_t)e < cnt[j]) ? __ldg(t.rkey + lo[j] + e) : EJ_NULL_KEY;
  }

  // 2. row prefixes: within the warp (probe order 32j + lane), then the block
  unsigned long long pre[PR_ITEMS];
  unsigned long long wrun = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const unsigned long long incl = ej_warp_inclusive_sum<unsigned long long>(cnt[j]);
    pre[j] = wrun + incl - cnt[j];
    wrun += __shfl_sync(EJ_FULL_MASK, incl, 31);
  }
  if (lane == 0) sm.wtot[warp] = wrun;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long x = lane < PR_WARPS ? sm.wtot[lane] : 0ull;
    const unsigned long long incl = ej_warp_inclusive_sum<unsigned long long>(x);
    if (lane < PR_WARPS) sm.woff[lane] = incl - x;
    const unsigned long long total = __shfl_sync(EJ_FULL_MASK, incl, 31);
    const unsigned long long off = ej_lookback_warp(lb_status, tile, total, st, 3u);
    if (lane == 0) {
      sm.tile_off = off;
      sm.total = total;
      if (last) {
        *d_total = off + total;
        if (off + total > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
      }
    }
  }
  __syncthreads();
  const unsigned long long gbase = sm.tile_off + sm.woff[warp];
  if (gbase >= cap) return;

  // 3. rows of this warp, 32 consecutive rows per round
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const unsigned long long a = __shfl_sync(EJ_FULL_MASK, pre[j], 0);
    const unsigned long long b = __shfl_sync(EJ_FULL_MASK, pre[j] + cnt[j], 31);
    for (unsigned long long o0 = a; o0 < b; o0 += 32) {
      const unsigned long long o = o0 + lane;
      // last lane whose first row is <= o (prefixes ascend with the lane)
      int src = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const unsigned long long x = __shfl_sync(EJ_FULL_MASK, pre[j], src + step);
        if (x <= o) src += step;
      }
      const uint32_t e = (uint32_t)(o - __shfl_sync(EJ_FULL_MASK, pre[j], src));
      const uint32_t rlo = __shfl_sync(EJ_FULL_MASK, lo[j], src);
      const int32_t sk = __shfl_sync(EJ_FULL_MASK, s[j].x, src);
      const int32_t sv = __shfl_sync(EJ_FULL_MASK, s[j].y, src);
      int32_t key = EJ_NULL_KEY;
#pragma unroll
      for (int q = 0; q < PW_PREFETCH; q++) {
        const int32_t kq = __shfl_sync(EJ_FULL_MASK, kk[j][q], src);
        if (e == (uint32_t)q) key = kq;
      }
      const bool valid = o < b;
      if (valid && e >= PW_PREFETCH) key = __ldg(t.rkey + rlo + e);
      const unsigned long long g = gbase + o;  // warp prefixes start at 0
      if (valid && g < cap) {
        const int32_t rv = rlo == NULL_RUN ? EJ_NULL_KEY : sv;
        __stcs(reinterpret_cast<int4*>(out + g), make_int4(key, rv, sk, sv));
      }
    }
  }
}
