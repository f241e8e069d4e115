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
//   3. one CTA per bucket orders the bucket by bits 0..15 in shared memory
//      (counting by bits 8..15, then each of the 256 sub-buckets by bits 0..7)
//      and writes the table's two columns rkey[]/rval[].
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
constexpr int LS_CAP = 3072;                 // rows of a bucket sorted in shared memory
constexpr int LS_PER = LS_CAP / LS_THREADS;  // rows per thread
constexpr uint32_t LS_SMALL = 32;            // sub-buckets up to this size: one thread's insertion sort

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
  uint2 row[LS_CAP];      // the bucket's tuples in sub-bucket order
  uint32_t hsh[LS_CAP];   // their hashes
  uint32_t cnt[256];      // counts of a digit, then running positions
  uint32_t start[257];    // sub-bucket starts
  uint32_t warp_tmp[LS_THREADS / 32 + 1];
  uint32_t nbig;
  uint32_t big[256];      // sub-buckets longer than LS_SMALL
  uint8_t isbig[256];
};

// exclusive sum of cnt[0..255] into dst[0..255] (dst[256] = total); every thread
__device__ __forceinline__ void ls_scan256(const uint32_t* cnt, uint32_t* dst, uint32_t* warp_tmp) {
  const uint32_t v = cnt[threadIdx.x];
  uint32_t total;
  const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(v, warp_tmp, &total);
  dst[threadIdx.x] = ex;
  if (threadIdx.x == 0) dst[256] = total;
  __syncthreads();
}

// The CTA sorts the rows [a, a + len) of `src` by hash bits 0..7 (all of them
// share bits 8..31) into rkey/rval at the same positions: a counting sort
// through global memory (order among equal hashes, which are equal keys,
// unspecified).  Shared counters: sm.cnt.
__device__ void ls_digit_global(LsSmem& sm, const ej_tuple* __restrict__ src, uint64_t a, uint32_t len,
                                int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  sm.cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint2* s2 = reinterpret_cast<const uint2*>(src);
  for (uint32_t j = threadIdx.x; j < len; j += LS_THREADS)
    atomicAdd(&sm.cnt[ej_hash32(s2[a + j].y) & 255u], 1u);
  __syncthreads();
  uint32_t c = sm.cnt[threadIdx.x];
  uint32_t total;
  const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(c, sm.warp_tmp, &total);
  sm.cnt[threadIdx.x] = ex;
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < len; j += LS_THREADS) {
    const uint2 x = s2[a + j];
    const uint32_t p = atomicAdd(&sm.cnt[ej_hash32(x.y) & 255u], 1u);
    rkey[a + p] = (int32_t)x.x;
    rval[a + p] = (int32_t)x.y;
  }
  __syncthreads();
}

// A bucket larger than shared memory: by bits 8..15 from `in` into `tmp`
// (same positions), then every sub-bucket by bits 0..7 into the columns.
__device__ void ls_bucket_global(LsSmem& sm, const ej_tuple* __restrict__ in, ej_tuple* __restrict__ tmp,
                                 uint64_t lo, uint32_t m, int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  const uint2* s2 = reinterpret_cast<const uint2*>(in);
  uint2* t2 = reinterpret_cast<uint2*>(tmp);
  sm.cnt[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < m; j += LS_THREADS) atomicAdd(&sm.cnt[(ej_hash32(s2[lo + j].y) >> 8) & 255u], 1u);
  __syncthreads();
  ls_scan256(sm.cnt, sm.start, sm.warp_tmp);
  sm.cnt[threadIdx.x] = sm.start[threadIdx.x];
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < m; j += LS_THREADS) {
    const uint2 x = s2[lo + j];
    const uint32_t p = atomicAdd(&sm.cnt[(ej_hash32(x.y) >> 8) & 255u], 1u);
    t2[lo + p] = x;
  }
  __syncthreads();  // the CTA's own global writes are visible to it past the barrier
  for (uint32_t s = 0; s < 256; s++) {
    const uint32_t a = sm.start[s], len = sm.start[s + 1] - a;
    if (len) ls_digit_global(sm, tmp, lo + a, len, rkey, rval);
  }
}

// One CTA per bucket b = top 16 hash bits: rows [bstart[b], bstart[b + 1]) of
// `in` (ordered by those bits) into the columns, ordered by the full hash.
__global__ void __launch_bounds__(LS_THREADS)
msd_local_kernel(const ej_tuple* __restrict__ in, ej_tuple* __restrict__ tmp, const uint32_t* __restrict__ bstart,
                 int32_t* __restrict__ rkey, int32_t* __restrict__ rval) {
  extern __shared__ __align__(16) unsigned char ls_smem_raw[];
  LsSmem& sm = *reinterpret_cast<LsSmem*>(ls_smem_raw);
  const uint32_t b = blockIdx.x;
  // bounds clamped to [0, n) and ordered (they are, unless a scan timed out)
  const uint32_t n = bstart[MSD_BUCKETS];
  const uint64_t lo = min(bstart[b], n);
  const uint32_t m = max(min(bstart[b + 1], n), (uint32_t)lo) - (uint32_t)lo;
  if (m == 0) return;
  if (m > (uint32_t)LS_CAP) {
    ls_bucket_global(sm, in, tmp, lo, m, rkey, rval);
    return;
  }
  const unsigned t = threadIdx.x;
  sm.cnt[t] = 0;
  sm.isbig[t] = 0;
  if (t == 0) sm.nbig = 0;
  __syncthreads();
  // 1. rows into registers (coalesced), ranked within their bits 8..15 digit
  const uint2* src = reinterpret_cast<const uint2*>(in) + lo;
  uint2 v[LS_PER];
  uint32_t h[LS_PER], rk[LS_PER];
#pragma unroll
  for (int i = 0; i < LS_PER; i++) {
    const uint32_t j = t + (uint32_t)i * LS_THREADS;
    if (j < m) {
      v[i] = __ldcs(src + j);
      h[i] = ej_hash32(v[i].y);
    }
  }
#pragma unroll
  for (int i = 0; i < LS_PER; i++)
    if (t + (uint32_t)i * LS_THREADS < m) rk[i] = atomicAdd(&sm.cnt[(h[i] >> 8) & 255u], 1u);
  __syncthreads();
  ls_scan256(sm.cnt, sm.start, sm.warp_tmp);
  // 2. every row to its sub-bucket
#pragma unroll
  for (int i = 0; i < LS_PER; i++)
    if (t + (uint32_t)i * LS_THREADS < m) {
      const uint32_t p = sm.start[(h[i] >> 8) & 255u] + rk[i];
      sm.row[p] = v[i];
      sm.hsh[p] = h[i];
    }
  __syncthreads();
  // 3. sub-bucket t by bits 0..7: insertion sort by one thread when short,
  //    else by the whole CTA below
  {
    const uint32_t a = sm.start[t], e = sm.start[t + 1];
    if (e - a <= LS_SMALL) {
      for (uint32_t i = a + 1; i < e; i++) {
        const uint32_t hk = sm.hsh[i];
        const uint2 rw = sm.row[i];
        uint32_t j = i;
        while (j > a && sm.hsh[j - 1] > hk) {
          sm.hsh[j] = sm.hsh[j - 1];
          sm.row[j] = sm.row[j - 1];
          j--;
        }
        sm.hsh[j] = hk;
        sm.row[j] = rw;
      }
    } else {
      sm.big[atomicAdd(&sm.nbig, 1u)] = t;
      sm.isbig[t] = 1;
    }
  }
  __syncthreads();
  // 4. the rows of short sub-buckets to the columns (coalesced)
  for (uint32_t k = t; k < m; k += LS_THREADS) {
    if (sm.isbig[(sm.hsh[k] >> 8) & 255u]) continue;
    const uint2 x = sm.row[k];
    rkey[lo + k] = (int32_t)x.x;
    rval[lo + k] = (int32_t)x.y;
  }
  // 5. long sub-buckets: a counting sort by bits 0..7, straight to the columns
  const uint32_t nbig = sm.nbig;
  for (uint32_t q = 0; q < nbig; q++) {
    const uint32_t s = sm.big[q];
    const uint32_t a = sm.start[s], len = sm.start[s + 1] - a;
    __syncthreads();
    sm.cnt[t] = 0;
    __syncthreads();
    for (uint32_t j = t; j < len; j += LS_THREADS) atomicAdd(&sm.cnt[sm.hsh[a + j] & 255u], 1u);
    __syncthreads();
    const uint32_t c = sm.cnt[t];
    uint32_t total;
    const uint32_t ex = ej_block_exclusive_sum<LS_THREADS, uint32_t>(c, sm.warp_tmp, &total);
    sm.cnt[t] = ex;
    __syncthreads();
    for (uint32_t j = t; j < len; j += LS_THREADS) {
      const uint32_t p = a + atomicAdd(&sm.cnt[sm.hsh[a + j] & 255u], 1u);
      const uint2 x = sm.row[a + j];
      rkey[lo + p] = (int32_t)x.x;
      rval[lo + p] = (int32_t)x.y;
    }
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
  EJ_CUDA(h, cudaFuncSetAttribute(msd_local_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LsSmem)));
  msd_local_kernel<<<MSD_BUCKETS, LS_THREADS, sizeof(LsSmem), h->stream>>>(tmp_b, tmp_a, bstart, rkey, rval);
  return ej_check_launch(h, "msd_local_kernel");
}
