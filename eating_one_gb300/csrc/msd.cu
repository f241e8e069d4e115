// msd.cu - the hash-sorted table build of large hash tables: two unordered
// most-significant-digit radix passes, then one shared-memory sort per bucket.
//
// The table (hash_join.cu) needs R ordered by hash32(val), with equal keys
// adjacent; the order among rows of one key is never used.  So no pass has to
// be stable, and the sort can go most-significant digit first:
//   1. an unordered radix pass by hash bits 24..31 (256 segments);
//   2. an unordered segmented pass by bits 16..23 inside every segment (65536
//      buckets of about |R|/65536 rows) - its tile descriptors are laid out on
//      the device from the first pass's offsets, so the host never waits;
//   3. one CTA per group of consecutive buckets (about 2048 rows) orders the
//      group by its remaining hash bits in shared memory (a counting pass by
//      12 of them into sub-buckets of a few rows, then every row ranked within
//      its sub-bucket) and writes each row once, to its place in the table's
//      two columns rkey[]/rval[].
// Three passes over R instead of the four of an LSD sort, none with the
// ballot ranking a stable pass needs.  A bucket too large for shared memory
// (many rows of few keys) is sorted by its CTA through global memory
// instead, one 8-bit digit at a time.
//
// Replaces, for the hash join's build side, the reference's partitioning of
// R (joins/hashJoin_gpu/main_street/partitioning.cu:133-271, rcount_partitioning
// + rpartitioning, one 6-bit digit per pass with a host round trip each).
#include "ej_device.cuh"
#include "msd.cuh"

namespace {

constexpr uint32_t MSD_BUCKET_BITS = 16;
constexpr uint32_t MSD_BUCKETS = 1u << MSD_BUCKET_BITS;
constexpr int LS_THREADS = 256;
constexpr int LS_CAP = 3072;                 // rows of a bucket group sorted in shared memory
constexpr int LS_PER = LS_CAP / LS_THREADS;  // rows per thread
constexpr uint32_t LS_ROWS = 2048;           // bucket groups aim at this many rows
constexpr uint32_t LS_DIGIT_BITS = 12;       // digit of the counting pass in shared memory
constexpr uint32_t LS_DIGITS = 1u << LS_DIGIT_BITS;
constexpr uint32_t LS_MAX_GROUP_BITS = 4;    // groups of at most 16 buckets
constexpr uint32_t LS_SMALL = 32;            // sub-buckets up to this size: each row ranked on its own

// the first pass's digit d (cells d * ntiles1 + t) is segment d: its start,
// its tiles, and the first tile of the second pass it gets
struct MsdSegments {
  uint32_t start[257];  // start[256] = n
  uint32_t end[256];    // start[d] + rows of segment d
  uint32_t tbase[257];  // first tile of the second pass; tbase[256] = tiles in use
};

__global__ void __launch_bounds__(256) msd_segments_kernel(const uint32_t* __restrict__ offs1, uint32_t ntiles1,
                                                           uint64_t n, MsdSegments* __restrict__ seg) {
  __shared__ uint32_t tmp[256 / 32 + 1];
  const uint32_t d = threadIdx.x;
  // clamped so that offsets left too small by a timed-out scan still give
  // ordered segments inside [0, n)
  const uint32_t s = min(offs1[(uint64_t)d * ntiles1], (uint32_t)n);
  const uint32_t e = max(s, d < 255 ? min(offs1[(uint64_t)(d + 1) * ntiles1], (uint32_t)n) : (uint32_t)n);
  const uint32_t tiles = (e - s + EJ_RX_TILE - 1) / EJ_RX_TILE;
  uint32_t total;
  const uint32_t base = ej_block_exclusive_sum<256, uint32_t>(tiles, tmp, &total);
  seg->start[d] = s;
  seg->tbase[d] = base;
  seg->end[d] = e;
  if (d == 255) {
    seg->start[256] = (uint32_t)n;
    seg->tbase[256] = total;
  }
}

// descriptor of every tile of the second pass: tile t of segment d covers
// rows start[d] + 4096 t ... and owns cells 256 tbase[d] + t + k tiles_d
// (digit k); tiles past those in use are empty and own cells past them all
__global__ void __launch_bounds__(256) msd_tiles_kernel(const MsdSegments* __restrict__ seg,
                                                        ej_rx_tile* __restrict__ desc, uint32_t max_tiles) {
  __shared__ uint32_t tb[257];
  for (uint32_t i = threadIdx.x; i < 257; i += blockDim.x) tb[i] = seg->tbase[i];
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= max_tiles) return;
  const uint32_t used = tb[256];
  ej_rx_tile t;
  t.src = nullptr;
  t.pad = 0;
  if (i < used) {
    uint32_t lo = 0, hi = 256;  // the segment d with tb[d] <= i < tb[d + 1]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (tb[mid] <= i) lo = mid; else hi = mid;
    }
    const uint32_t d = lo, k = i - tb[d], tiles = tb[d + 1] - tb[d];
    const uint32_t s = seg->start[d] + k * EJ_RX_TILE, e = seg->end[d];
    t.start = s;
    t.n = min((uint32_t)EJ_RX_TILE, e - s);
    t.cell0 = 256u * tb[d] + k;
    t.stride = tiles;
  } else {
    t.start = 0;
    t.n = 0;
    t.cell0 = 256u * i;  // i >= used: past every cell of the tiles in use
    t.stride = 1;
  }
  desc[i] = t;
}

// bucket (d1, d2) starts where the second pass put digit d2 of segment d1's
// first tile; bstart[65536] = n
__global__ void __launch_bounds__(256) msd_bucket_kernel(const MsdSegments* __restrict__ seg,
                                                         const uint32_t* __restrict__ offs2, uint64_t n,
                                                         uint32_t* __restrict__ bstart) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > MSD_BUCKETS) return;
  if (b == MSD_BUCKETS) {
    bstart[b] = (uint32_t)n;
    return;
  }
  const uint32_t d1 = b >> 8, d2 = b & 255u;
  const uint32_t tiles = seg->tbase[d1 + 1] - seg->tbase[d1];
  bstart[b] = tiles ? offs2[256ull * seg->tbase[d1] + (uint64_t)d2 * tiles] : seg->start[d1];
}

struct LsSmem {
  uint2 row[LS_CAP];              // the group's tuples in digit order
  uint32_t hsh[LS_CAP];           // their hashes
  uint32_t cnt[LS_DIGITS + 1];    // digit counts, then digit starts (cnt[LS_DIGITS] = rows)
  uint32_t cnt2[256];             // counts of a long sub-bucket's remaining bits (at most 8 of them)
  uint32_t big[LS_CAP / (LS_SMALL + 1) + 1];  // digits whose sub-bucket is longer than LS_SMALL
  uint32_t warp_tmp[LS_THREADS / 32 + 1];
  uint32_t nbig;
};

// Digit d's counter sits at ls_at(d) = d ^ ((d >> 5) & 31), a permutation
// within each 32-counter row: the scan below, where thread t takes digits
// 16t .. 16t + 15, and the placement, where a warp's lanes take consecutive
// rows of non-decreasing digits, both read 32 distinct banks per instruction
// (a plain layout gave the scan 16-way conflicts).  Index LS_DIGITS (the
// total) maps to itself.
__device__ __forceinline__ uint32_t ls_at(uint32_t d) { return d ^ ((d >> 5) & 31u); }

// exclusive sum in place of the LS_DIGITS counters (at ls_at(d)); c at
// LS_DIGITS = total.  Every thread, LS_DIGITS / LS_THREADS consecutive
// digits; the counters are read twice rather than held, as the caller's rows
// occupy the registers
__device__ __forceinline__ void ls_scan_digits(uint32_t* c, uint32_t* warp_tmp) {
  constexpr int PER = LS_DIGITS / LS_THREADS;
  const uint32_t d0 = threadIdx.x * PER;
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < PER; i++) sum += c[ls_at(d0 + i)];
  uint32_t total;
  uint32_t run = ej_block_exclusive_sum<LS_THREADS, uint32_t>(sum, warp_tmp, &total);
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const uint32_t x = c[ls_at(d0 + i)];
    c[ls_at(d0 + i)] = run;
    run += x;
  }
  if (threadIdx.x == 0) c[LS_DIGITS] = total;
  __syncthreads();
}

// The CTA sorts the rows [a, a + len) of `src` by hash bits 0..7 (all of them
// share bits 8..31) into rkey/rval at the same positions: a counting sort
// through global memory (order among equal hashes, which are equal keys,
// unspecified).  Shared counters: sm.cnt2.  `src` was written earlier in this
// launch (by this CTA), so it is read through L2 (__ldcg), never through the
// read-only cache, which another CTA on the SM may have filled with the same
// lines before they were written; a stale line would make the two loops
// below see different rows.
__device__ void ls_digit_global(LsSmem& sm, const ej_tuple* src, uint64_t a, uint32_t len,
                                int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  sm.cnt2[threadIdx.x] = 0;
  __syncthreads();
  const uint2* s2 = reinterpret_cast<const uint2*>(src);
  for (uint32_t j = threadIdx.x; j < len; j += LS_THREADS)
    atomicAdd(&sm.cnt2[ej_hash32(__ldcg(s2 + a + j).y) & 255u], 1u);
  __syncthreads();
  uint32_t c = sm.cnt2[threadIdx.x];
  uint32_t total;
  const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(c, sm.warp_tmp, &total);
  sm.cnt2[threadIdx.x] = ex;
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < len; j += LS_THREADS) {
    const uint2 x = __ldcg(s2 + a + j);
    const uint32_t p = atomicAdd(&sm.cnt2[ej_hash32(x.y) & 255u], 1u);
    if (p < len) {  // always; a guard that keeps every store inside the range
      rkey[a + p] = (int32_t)x.x;
      rval[a + p] = (int32_t)x.y;
    }
  }
  __syncthreads();
}

// A bucket larger than shared memory: by bits 8..15 from `in` into `tmp`
// (same positions), then every sub-bucket by bits 0..7 into the columns.
// Shared counters: sm.cnt (256 of them, with their starts in cnt[256 ...]).
__device__ void ls_bucket_global(LsSmem& sm, const ej_tuple* __restrict__ in, ej_tuple* __restrict__ tmp,
                                 uint64_t lo, uint32_t m, int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  const uint2* s2 = reinterpret_cast<const uint2*>(in);
  uint2* t2 = reinterpret_cast<uint2*>(tmp);
  uint32_t* cur = sm.cnt;
  uint32_t* st = sm.cnt + 256;  // 257 starts
  cur[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < m; j += LS_THREADS) atomicAdd(&cur[(ej_hash32(s2[lo + j].y) >> 8) & 255u], 1u);
  __syncthreads();
  {
    const uint32_t c = cur[threadIdx.x];
    uint32_t total;
    const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(c, sm.warp_tmp, &total);
    st[threadIdx.x] = ex;
    cur[threadIdx.x] = ex;
    if (threadIdx.x == 0) st[256] = total;
    __syncthreads();
  }
  for (uint32_t j = threadIdx.x; j < m; j += LS_THREADS) {
    const uint2 x = s2[lo + j];
    const uint32_t p = atomicAdd(&cur[(ej_hash32(x.y) >> 8) & 255u], 1u);
    if (p < m) t2[lo + p] = x;  // always; a guard that keeps every store inside the range
  }
  __syncthreads();  // the CTA's own global writes are visible to it past the barrier
  for (uint32_t s = 0; s < 256; s++) {
    const uint32_t a = st[s], len = st[s + 1] - a;
    if (len) ls_digit_global(sm, tmp, lo + a, len, rkey, rval);
  }
}

// The CTA sorts the m <= LS_CAP rows [lo, lo + m) of `in`, which share hash
// bits low_bits..31 (LS_DIGIT_BITS <= low_bits <= LS_DIGIT_BITS + 8), into the
// columns by the full hash: a counting pass by the LS_DIGIT_BITS bits below
// low_bits groups the rows into sub-buckets of a few rows each; every row's
// place in its sub-bucket is the number of rows there with a smaller hash
// (or the same hash and an earlier slot), so each row is written once, at
// its final position.  Long sub-buckets (many rows of few keys) are sorted
// by the whole CTA instead: a counting sort by their remaining bits.
//
// PER: row slots per thread (m <= PER * LS_THREADS), so that a small group
// does not pay for the slots of the largest; up to 9 slots the rows' hashes
// stay in registers between the ranking and the placement (beyond that they
// are computed again, for want of registers).
template <int PER>
__device__ void ls_sort_smem(LsSmem& sm, const ej_tuple* __restrict__ in, uint64_t lo, uint32_t m,
                             uint32_t low_bits, int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  constexpr bool KEEP = PER <= 9;
  const unsigned t = threadIdx.x;
  const uint32_t sh = low_bits - LS_DIGIT_BITS;  // bits under the digit
  for (uint32_t i = t; i < LS_DIGITS / 4; i += LS_THREADS) reinterpret_cast<uint4*>(sm.cnt)[i] = make_uint4(0, 0, 0, 0);
  if (t == 0) sm.nbig = 0;
  __syncthreads();
  // 1. rows into registers (coalesced), ranked within their digit
  const uint2* src = reinterpret_cast<const uint2*>(in) + lo;
  uint2 v[PER];
  uint32_t rk[PER], hk[KEEP ? PER : 1];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const uint32_t j = t + (uint32_t)i * LS_THREADS;
    if (j < m) v[i] = __ldcs(src + j);
  }
#pragma unroll
  for (int i = 0; i < PER; i++)
    if (t + (uint32_t)i * LS_THREADS < m) {
      const uint32_t hv = ej_hash32(v[i].y);
      if (KEEP) hk[KEEP ? i : 0] = hv;
      rk[i] = atomicAdd(&sm.cnt[ls_at((hv >> sh) & (LS_DIGITS - 1))], 1u);
    }
  __syncthreads();
  ls_scan_digits(sm.cnt, sm.warp_tmp);
  // 2. every row to its digit's sub-bucket
#pragma unroll
  for (int i = 0; i < PER; i++)
    if (t + (uint32_t)i * LS_THREADS < m) {
      const uint32_t hv = KEEP ? hk[KEEP ? i : 0] : ej_hash32(v[i].y);
      const uint32_t p = sm.cnt[ls_at((hv >> sh) & (LS_DIGITS - 1))] + rk[i];
      sm.row[p] = v[i];
      sm.hsh[p] = hv;
    }
  __syncthreads();
  // 3. each row of a short sub-bucket straight to its place (the lanes of a
  //    warp take consecutive slots, so their stores stay within a few rows
  //    of each other); long sub-buckets are listed for step 4
  for (uint32_t p = t; p < m; p += LS_THREADS) {
    const uint32_t hv = sm.hsh[p];
    const uint32_t d = (hv >> sh) & (LS_DIGITS - 1);
    const uint32_t a = sm.cnt[ls_at(d)], e = sm.cnt[ls_at(d + 1)];
    if (e - a > LS_SMALL) {
      if (p == a) sm.big[atomicAdd(&sm.nbig, 1u)] = d;
      continue;
    }
    uint32_t r = a;
    for (uint32_t q = a; q < e; q++) {
      const uint32_t x = sm.hsh[q];
      r += (x < hv || (x == hv && q < p)) ? 1u : 0u;
    }
    const uint2 row = sm.row[p];
    rkey[lo + r] = (int32_t)row.x;
    rval[lo + r] = (int32_t)row.y;
  }
  __syncthreads();
  // 4. long sub-buckets: a counting sort by the bits under the digit,
  //    straight to the columns
  const uint32_t nbig = sm.nbig, rmask = (1u << sh) - 1u;
  for (uint32_t q = 0; q < nbig; q++) {
    const uint32_t d = sm.big[q];
    const uint32_t a = sm.cnt[ls_at(d)], len = sm.cnt[ls_at(d + 1)] - a;
    sm.cnt2[t] = 0;
    __syncthreads();
    for (uint32_t j = t; j < len; j += LS_THREADS) atomicAdd(&sm.cnt2[sm.hsh[a + j] & rmask], 1u);
    __syncthreads();
    const uint32_t c = sm.cnt2[t];
    uint32_t total;
    const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(c, sm.warp_tmp, &total);
    sm.cnt2[t] = ex;
    __syncthreads();
    for (uint32_t j = t; j < len; j += LS_THREADS) {
      const uint2 x = sm.row[a + j];
      const uint32_t p = a + atomicAdd(&sm.cnt2[sm.hsh[a + j] & rmask], 1u);
      rkey[lo + p] = (int32_t)x.x;
      rval[lo + p] = (int32_t)x.y;
    }
    __syncthreads();
  }
  __syncthreads();  // shared memory is reused by the caller's next range
}

// ls_sort_smem with the fewest row slots per thread that hold m rows (groups
// aim at LS_ROWS = 8 slots' worth; 9 takes most of those a little over)
__device__ __forceinline__ void ls_sort_rows(LsSmem& sm, const ej_tuple* __restrict__ in, uint64_t lo, uint32_t m,
                                             uint32_t low_bits, int32_t* __restrict__ rkey,
                                             int32_t* __restrict__ rval) {
  if (m <= 4u * LS_THREADS)
    ls_sort_smem<4>(sm, in, lo, m, low_bits, rkey, rval);
  else if (m <= 8u * LS_THREADS)
    ls_sort_smem<8>(sm, in, lo, m, low_bits, rkey, rval);
  else if (m <= 9u * LS_THREADS)
    ls_sort_smem<9>(sm, in, lo, m, low_bits, rkey, rval);
  else
    ls_sort_smem<LS_PER>(sm, in, lo, m, low_bits, rkey, rval);
}

// One CTA per group of 2^g consecutive buckets (b = top 16 hash bits), whose
// rows [bstart[b0], bstart[b0 + 2^g]) of `in` share hash bits 16 + g .. 31:
// into the columns ordered by the full hash.  A group larger than shared
// memory goes bucket by bucket, and a bucket larger than shared memory
// through global memory.
__global__ void __launch_bounds__(LS_THREADS, 4)
msd_local_kernel(const ej_tuple* __restrict__ in, ej_tuple* __restrict__ tmp, const uint32_t* __restrict__ bstart,
                 uint32_t g, int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  extern __shared__ __align__(16) unsigned char ls_smem_raw[];
  LsSmem& sm = *reinterpret_cast<LsSmem*>(ls_smem_raw);
  // bounds clamped to [0, n) and ordered (they are, unless a scan timed out)
  const uint32_t n = bstart[MSD_BUCKETS];
  const uint32_t b0 = blockIdx.x << g, b1 = b0 + (1u << g);
  const uint32_t lo = min(bstart[b0], n);
  const uint32_t hi = max(min(bstart[b1], n), lo);
  if (hi - lo <= (uint32_t)LS_CAP) {
    if (hi > lo) ls_sort_rows(sm, in, lo, hi - lo, MSD_BUCKET_BITS + g, rkey, rval);
    return;
  }
  for (uint32_t b = b0; b < b1; b++) {
    const uint32_t blo = max(min(bstart[b], n), lo);
    const uint32_t bhi = min(max(min(bstart[b + 1], n), blo), hi);
    if (bhi - blo > (uint32_t)LS_CAP)
      ls_bucket_global(sm, in, tmp, blo, bhi - blo, rkey, rval);
    else if (bhi > blo)
      ls_sort_rows(sm, in, blo, bhi - blo, MSD_BUCKET_BITS, rkey, rval);
  }
}

}  // namespace

void ej_msd_plan_add(ej_plan_bytes& p, ej_msd_plan& mp, uint64_t n) {
  mp.n = n;
  ej_radix_plan_add(p, mp.pass1, n);
  // the second pass: at most one partial tile more per segment
  mp.pass2.n = n;
  mp.pass2.ntiles = ej_radix_tiles(n) + 256;
  const uint64_t cells = (uint64_t)mp.pass2.ntiles * 256;
  mp.pass2.hist_off = p.add(cells * sizeof(uint32_t));
  mp.pass2.offs_off = p.add((cells + 1) * sizeof(uint32_t));
  mp.pass2.scan_off = p.add(ej_scan_scratch_bytes(cells));
  mp.desc_off = p.add((size_t)mp.pass2.ntiles * sizeof(ej_rx_tile));
  mp.seg_off = p.add(sizeof(MsdSegments));
  mp.bstart_off = p.add((MSD_BUCKETS + 1) * sizeof(uint32_t));
}

ej_status ej_msd_sort(ej_handle* h, const ej_msd_plan& mp, const ej_tuple* R, ej_tuple* tmp_a, ej_tuple* tmp_b,
                      int32_t* rkey, int32_t* rval) {
  if (mp.n == 0) return EJ_OK;
  if (mp.n >= 0xFFFFFFFFull) return ej_fail(h, EJ_ERR_TOO_LARGE, "table of %llu rows", (unsigned long long)mp.n);
  // 1. by bits 24..31
  EJ_TRY(ej_partition_pass(h, mp.pass1, R, tmp_a, 24u, 8u, EJ_DIGIT_HASH));
  // 2. by bits 16..23 inside every segment, tiles laid out on the device
  MsdSegments* seg = reinterpret_cast<MsdSegments*>(ej_arena_at(h, mp.seg_off));
  ej_rx_tile* desc = reinterpret_cast<ej_rx_tile*>(ej_arena_at(h, mp.desc_off));
  const uint32_t* offs1 = reinterpret_cast<const uint32_t*>(ej_arena_at(h, mp.pass1.offs_off));
  msd_segments_kernel<<<1, 256, 0, h->stream>>>(offs1, mp.pass1.ntiles, mp.n, seg);
  EJ_TRY(ej_check_launch(h, "msd_segments_kernel"));
  msd_tiles_kernel<<<(mp.pass2.ntiles + 255) / 256, 256, 0, h->stream>>>(seg, desc, mp.pass2.ntiles);
  EJ_TRY(ej_check_launch(h, "msd_tiles_kernel"));
  ej_radix_plan p2 = mp.pass2;
  p2.tiles = desc;
  EJ_TRY(ej_partition_pass(h, p2, tmp_a, tmp_b, 16u, 8u, EJ_DIGIT_HASH));
  // 3. bucket bounds, then every bucket by bits 0..15 into the columns
  uint32_t* bstart = reinterpret_cast<uint32_t*>(ej_arena_at(h, mp.bstart_off));
  const uint32_t* offs2 = reinterpret_cast<const uint32_t*>(ej_arena_at(h, mp.pass2.offs_off));
  msd_bucket_kernel<<<(MSD_BUCKETS + 1 + 255) / 256, 256, 0, h->stream>>>(seg, offs2, mp.n, bstart);
  EJ_TRY(ej_check_launch(h, "msd_bucket_kernel"));
  // groups of 2^g buckets of about LS_ROWS rows in all
  uint32_t g = 0;
  while (g < LS_MAX_GROUP_BITS && ((uint64_t)LS_ROWS << MSD_BUCKET_BITS) >= (mp.n << (g + 1))) g++;
  EJ_CUDA(h, cudaFuncSetAttribute(msd_local_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LsSmem)));
  msd_local_kernel<<<MSD_BUCKETS >> g, LS_THREADS, sizeof(LsSmem), h->stream>>>(tmp_b, tmp_a, bstart, g, rkey, rval);
  return ej_check_launch(h, "msd_local_kernel");
}
