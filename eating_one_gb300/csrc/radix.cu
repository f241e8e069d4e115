// radix.cu - stable radix partitioning of TUPLE arrays by hash digits.
//
// Replaces the reference's radix partitioner (joins/hashJoin_gpu/main_street/
// partitioning.cu:15-271 lcount/rcount_partitioning + lpartitioning/
// rpartitioning, driven by hj.cc:430-534 and :702-829): 16-thread blocks that
// each walk 256 consecutive tuples, one 6-bit digit per pass, a host
// round-trip per pass.  Here one pass is three launches on the stream:
//   1. rx_hist_kernel    per 4096-tuple tile, digit counts in warp-private
//                        shared-memory histograms, stored digit-major:
//                        hist[digit * ntiles + tile];
//   2. look-back scan    of the digit-major histogram gives every (digit, tile)
//                        its global output offset (scan.cu);
//   3. rx_scatter_kernel stages the tile in shared memory, ranks it stably by
//                        digit (warp-ordered ranking; the lanes sharing a
//                        digit come from one ballot per digit bit), and writes
//                        it digit run by digit run, so consecutive threads
//                        store consecutive addresses.
// Digits are up to 8 bits of hash32(val).  Positions are 32-bit: n < 2^32.
#include "ej_device.cuh"

namespace {

constexpr int RX_THREADS = 256;
constexpr int RX_WARPS = RX_THREADS / 32;
constexpr int RX_TILE = (int)EJ_RX_TILE;
constexpr int RX_WARP_SPAN = RX_TILE / RX_WARPS;  // consecutive tuples per warp
constexpr int RX_ROUNDS = RX_WARP_SPAN / 32;      // 32
constexpr int RX_MAX_DIGITS = 256;

template <int KIND>
__device__ __forceinline__ uint32_t rx_digit(int32_t val, uint32_t shift, uint32_t mask) {
  const uint32_t key = KIND == EJ_DIGIT_HASH ? ej_hash32((uint32_t)val) : ((uint32_t)val ^ 0x80000000u);
  return (key >> shift) & mask;
}

// The tile of this block: uniform EJ_RX_TILE-row tiles of one relation (tiles ==
// nullptr; histogram cell of digit d = d * ntiles + tile), or one entry of a
// descriptor array whose tiles never cross a segment (batched joins).
struct RxTile {
  const ej_tuple* base;  // the tile's first input row
  uint32_t n, cell0, stride;
};

// SRC: the descriptors carry their tiles' source rows (a pass over inputs
// that lie in separate arrays)
template <bool SRC>
__device__ __forceinline__ RxTile rx_tile(const ej_tuple* in, const ej_rx_tile* tiles, uint64_t n,
                                          uint32_t ntiles) {
  RxTile t;
  if (tiles) {
    const ej_rx_tile& d = tiles[blockIdx.x];
    t.base = SRC ? d.src : in + d.start;
    t.n = d.n;
    t.cell0 = d.cell0;
    t.stride = d.stride;
  } else {
    const uint64_t start = (uint64_t)blockIdx.x * RX_TILE;
    t.base = in + start;
    t.n = (uint32_t)min((uint64_t)RX_TILE, n - start);
    t.cell0 = blockIdx.x;
    t.stride = ntiles;
  }
  return t;
}

template <int KIND, bool SRC = false>
__global__ void __launch_bounds__(RX_THREADS)
rx_hist_kernel(const ej_tuple* __restrict__ in, uint64_t n, const ej_rx_tile* __restrict__ tiles,
               uint32_t* __restrict__ hist, uint32_t ntiles, uint32_t shift, uint32_t mask) {
  __shared__ uint32_t cnt[RX_WARPS][RX_MAX_DIGITS];
  const uint32_t ndig = mask + 1u;
  for (int i = threadIdx.x; i < RX_WARPS * RX_MAX_DIGITS; i += RX_THREADS) (&cnt[0][0])[i] = 0u;
  __syncthreads();
  const RxTile tl = rx_tile<SRC>(in, tiles, n, ntiles);
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t wbase = warp * RX_WARP_SPAN;
  const int* vals = reinterpret_cast<const int*>(tl.base) + 1;  // .val of the tile's tuple i at vals[2*i]
  int v[RX_ROUNDS];
#pragma unroll
  for (int r = 0; r < RX_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    v[r] = i < tl.n ? __ldcs(vals + 2 * (uint64_t)i) : 0;
  }
  // warp-private histograms: counting order does not matter, so plain
  // shared-memory atomics (same-digit lanes of one instruction serialise in hardware)
#pragma unroll
  for (int r = 0; r < RX_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    if (i < tl.n) atomicAdd(&cnt[warp][rx_digit<KIND>(v[r], shift, mask)], 1u);
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < ndig; d += RX_THREADS) {
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < RX_WARPS; w++) t += cnt[w][d];
    hist[tl.cell0 + (uint64_t)d * tl.stride] = t;
  }
}

struct RxScatterSmem {
  ej_tuple sorted[RX_TILE];                // 32 KB: the tile in digit order
  uint32_t cnt[RX_WARPS][RX_MAX_DIGITS];   // per-warp digit counters, then bases
  uint32_t gbase[RX_MAX_DIGITS];
  uint32_t warp_tmp[RX_WARPS + 1];
};

// SOA: write the key and val of each tuple to two separate arrays (the last
// pass of a table build) instead of tuples.  STABLE false: the order within a
// digit's run is left to shared-memory atomics (a one-pass partition, where no
// later pass depends on it), which takes about a fifth of the ranking's
// instructions
template <int KIND, bool SOA, bool STABLE, bool SRC = false>
__global__ void __launch_bounds__(RX_THREADS, 4)
rx_scatter_kernel(const ej_tuple* __restrict__ in, uint64_t n, const ej_rx_tile* __restrict__ tiles,
                  ej_tuple* __restrict__ out, int32_t* __restrict__ out_keys, int32_t* __restrict__ out_vals,
                  const uint32_t* __restrict__ offs, uint32_t ntiles, uint32_t shift, uint32_t mask) {
  extern __shared__ __align__(16) unsigned char rx_smem_raw[];
  RxScatterSmem& sm = *reinterpret_cast<RxScatterSmem*>(rx_smem_raw);
  const uint32_t ndig = mask + 1u;
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const RxTile tl = rx_tile<SRC>(in, tiles, n, ntiles);
  const uint32_t tile_n = tl.n;
  for (int i = threadIdx.x; i < RX_WARPS * RX_MAX_DIGITS; i += RX_THREADS) (&sm.cnt[0][0])[i] = 0u;
  // unordered passes: the digit's global offset (thread d) is loaded now, so
  // that it is in hand when the ranking is done (the stable ranking has no
  // register to spare for it and loads it afterwards)
  uint32_t goff = 0;
  if (!STABLE && threadIdx.x < ndig) goff = offs[tl.cell0 + (uint64_t)threadIdx.x * tl.stride];

  // 1. the warp's RX_ROUNDS x 32 consecutive tuples into registers (coalesced,
  //    streaming: read once)
  const uint32_t wbase = warp * RX_WARP_SPAN;
  const uint2* src = reinterpret_cast<const uint2*>(tl.base);
  uint2 tup[RX_ROUNDS];
#pragma unroll
  for (int r = 0; r < RX_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    tup[r] = i < tile_n ? __ldcs(src + i) : make_uint2(0u, 0u);
  }
  __syncthreads();  // counters zeroed

  // 2. stable rank within the warp: round order, then lane order; the lanes
  //    sharing a digit come from one ballot per digit bit, the warp's running
  //    count of each digit from its shared-memory counter.  Each item keeps
  //    (digit << 16 | rank within the warp's items of that digit).
  uint32_t packed[RX_ROUNDS];
#pragma unroll
  for (int r = 0; r < RX_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    const bool valid = i < tile_n;
    const uint32_t d = valid ? rx_digit<KIND>((int32_t)tup[r].y, shift, mask) : 0u;
    if (!STABLE) {
      packed[r] = valid ? (d << 16) | atomicAdd(&sm.cnt[warp][d], 1u) : 0xFFFFFFFFu;
      continue;
    }
    const unsigned int peers = ej_match_digit<8>(d, __ballot_sync(EJ_FULL_MASK, valid));
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (valid && (int)lane == leader) {
      old = sm.cnt[warp][d];
      sm.cnt[warp][d] = old + __popc(peers);
    }
    old = __shfl_sync(EJ_FULL_MASK, old, leader < 0 ? 0 : leader);
    packed[r] = valid ? (d << 16) | (old + __popc(peers & ej_lanemask_lt())) : 0xFFFFFFFFu;
    __syncwarp();
  }
  __syncthreads();

  // 3. per digit: warp bases within the digit, the digit's start in the tile
  //    (cnt[w][d] becomes the tile position of warp w's first item of digit
  //    d) and the global base of the digit's run
  uint32_t total = 0;
  if (threadIdx.x < ndig) {
    const uint32_t d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < RX_WARPS; w++) {
      const uint32_t c = sm.cnt[w][d];
      sm.cnt[w][d] = total;
      total += c;
    }
  }
  uint32_t all;
  const uint32_t dstart = ej_block_exclusive_sum<RX_THREADS, uint32_t>(total, sm.warp_tmp, &all);
  if (threadIdx.x < ndig) {
    const uint32_t d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < RX_WARPS; w++) sm.cnt[w][d] += dstart;
    if (STABLE) goff = offs[tl.cell0 + (uint64_t)d * tl.stride];
    sm.gbase[d] = goff - dstart;
  }
  __syncthreads();

  // 4. every item to its sorted position in shared memory
#pragma unroll
  for (int r = 0; r < RX_ROUNDS; r++) {
    if (packed[r] != 0xFFFFFFFFu) {
      const uint32_t d = packed[r] >> 16;
      const uint32_t pos = sm.cnt[warp][d] + (packed[r] & 0xFFFFu);
      reinterpret_cast<uint2*>(sm.sorted)[pos] = tup[r];
    }
  }
  __syncthreads();

  // 5. write digit runs: sorted position k goes to gbase[digit] + k
  for (uint32_t k = threadIdx.x; k < tile_n; k += RX_THREADS) {
    const uint2 t = reinterpret_cast<const uint2*>(sm.sorted)[k];
    const uint32_t pos = sm.gbase[rx_digit<KIND>((int32_t)t.y, shift, mask)] + k;
    if (SOA) {
      out_keys[pos] = (int32_t)t.x;
      out_vals[pos] = (int32_t)t.y;
    } else {
      reinterpret_cast<uint2*>(out)[pos] = t;
    }
  }
}

}  // namespace

uint32_t ej_radix_tiles(uint64_t n) { return (uint32_t)((n + RX_TILE - 1) / RX_TILE); }

void ej_radix_plan_add(ej_plan_bytes& p, ej_radix_plan& rp, uint64_t n) {
  rp.n = n;
  rp.ntiles = ej_radix_tiles(n);
  const uint64_t cells = (uint64_t)rp.ntiles * RX_MAX_DIGITS;
  rp.hist_off = p.add(cells * sizeof(uint32_t));
  rp.offs_off = p.add((cells + 1) * sizeof(uint32_t));
  rp.scan_off = p.add(ej_scan_scratch_bytes(cells));
}

template <int KIND, bool SOA, bool STABLE = true, bool SRC = false>
static ej_status radix_pass_kind(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, ej_tuple* out,
                                 int32_t* out_keys, int32_t* out_vals, uint32_t shift, uint32_t bits) {
  const uint32_t mask = (1u << bits) - 1u;
  // uniform tiles use cells d * ntiles + tile; segmented tiles carry their own
  // cells, laid out segment by segment with a stride of the segment's tiles
  const uint64_t cells = rp.tiles ? (uint64_t)rp.ntiles * RX_MAX_DIGITS : (uint64_t)rp.ntiles << bits;
  uint32_t* hist = reinterpret_cast<uint32_t*>(ej_arena_at(h, rp.hist_off));
  uint32_t* offs = reinterpret_cast<uint32_t*>(ej_arena_at(h, rp.offs_off));
  if (rp.tiles && bits != 8) return ej_fail(h, EJ_ERR_INTERNAL, "segmented radix passes use 8-bit digits");
  rx_hist_kernel<KIND, SRC><<<rp.ntiles, RX_THREADS, 0, h->stream>>>(in, rp.n, rp.tiles, hist, rp.ntiles, shift,
                                                                     mask);
  EJ_TRY(ej_check_launch(h, "rx_hist_kernel"));
  EJ_TRY(ej_scan_u32_u32(h, hist, cells, offs, ej_arena_at(h, rp.scan_off)));
  EJ_CUDA(h, cudaFuncSetAttribute(rx_scatter_kernel<KIND, SOA, STABLE, SRC>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RxScatterSmem)));
  rx_scatter_kernel<KIND, SOA, STABLE, SRC><<<rp.ntiles, RX_THREADS, sizeof(RxScatterSmem), h->stream>>>(
      in, rp.n, rp.tiles, out, out_keys, out_vals, offs, rp.ntiles, shift, mask);
  return ej_check_launch(h, "rx_scatter_kernel");
}

static ej_status check_digit(ej_handle* h, uint32_t shift, uint32_t bits) {
  if (bits == 0 || bits > 8 || shift + bits > 32)
    return ej_fail(h, EJ_ERR_INTERNAL, "radix pass: bad digit (shift %u, bits %u)", shift, bits);
  return EJ_OK;
}

ej_status ej_radix_pass(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, ej_tuple* out,
                        uint32_t shift, uint32_t bits, int digit_kind) {
  if (rp.n == 0) return EJ_OK;
  EJ_TRY(check_digit(h, shift, bits));
  if (digit_kind == EJ_DIGIT_VALUE)
    return radix_pass_kind<EJ_DIGIT_VALUE, false>(h, rp, in, out, nullptr, nullptr, shift, bits);
  return radix_pass_kind<EJ_DIGIT_HASH, false>(h, rp, in, out, nullptr, nullptr, shift, bits);
}

ej_status ej_radix_pass_soa(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, int32_t* out_keys,
                            int32_t* out_vals, uint32_t shift, uint32_t bits, int digit_kind) {
  if (rp.n == 0) return EJ_OK;
  EJ_TRY(check_digit(h, shift, bits));
  if (digit_kind == EJ_DIGIT_VALUE)
    return radix_pass_kind<EJ_DIGIT_VALUE, true>(h, rp, in, nullptr, out_keys, out_vals, shift, bits);
  return radix_pass_kind<EJ_DIGIT_HASH, true>(h, rp, in, nullptr, out_keys, out_vals, shift, bits);
}

ej_status ej_partition_pass(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, ej_tuple* out,
                            uint32_t shift, uint32_t bits, int digit_kind) {
  if (rp.n == 0) return EJ_OK;
  EJ_TRY(check_digit(h, shift, bits));
  if (digit_kind == EJ_DIGIT_VALUE)
    return radix_pass_kind<EJ_DIGIT_VALUE, false, false>(h, rp, in, out, nullptr, nullptr, shift, bits);
  return radix_pass_kind<EJ_DIGIT_HASH, false, false>(h, rp, in, out, nullptr, nullptr, shift, bits);
}

ej_status ej_partition_pass_src(ej_handle* h, const ej_radix_plan& rp, ej_tuple* out, uint32_t shift,
                                uint32_t bits) {
  if (rp.n == 0) return EJ_OK;
  EJ_TRY(check_digit(h, shift, bits));
  if (!rp.tiles) return ej_fail(h, EJ_ERR_INTERNAL, "a pass over separate inputs needs tile descriptors");
  return radix_pass_kind<EJ_DIGIT_HASH, false, false, true>(h, rp, nullptr, out, nullptr, nullptr, shift, bits);
}
