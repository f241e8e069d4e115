// hash_join.cu - the table build and the probe (count with run descriptors,
// scan, write) shared by every join that probes R.
//
// Reference path replaced (joins/hashJoin_gpu/main_street): radix-partition
// both relations into ~|R|/64 partitions, split left partitions into 256-tuple
// chunks on the host, then `count` and `join` compare every chunk tuple with
// every tuple of the matching right partition (join_gpu.cu:9-113) - O(256*|Rp|)
// compares per block, and the write pass repeats all of them.
//
// Here:
//   build  R is sorted by hash32(val): tables of 2^20 rows and more by two
//          unordered MSD passes and a shared-memory sort per 16-bit bucket
//          (msd.cu), smaller ones and sorted indexes by four 8-bit LSD radix
//          passes (radix.cu); either writes it as two arrays rkey[]/rval[],
//          and start[b] marks where bucket b (top hb hash bits) begins - the
//          grouped layout of the reference's hash index (Bucket + Buck_array,
//          joins/CPU_JOIN/inner_cpu/inner-idx-bnlj.cc:142-166), built on the
//          device.  The hash is a bijection, so equal keys are one contiguous
//          run and a probe yields (run start, run length).
//   S      when the table does not fit in L2, S is radix-partitioned once by
//          the top pb hash bits, so consecutive probe tiles touch one table
//          region at a time and hit L2; otherwise S is probed in place.
//   probe  three launches per join (probe_write.cuh): a count pass finds
//          every probe's run and stores its descriptor (run start, length)
//          and each 128-probe warp tile's row total; a scan of the totals
//          gives every warp tile its output offset; the write pass reads the
//          probes with their descriptors, fetches the run keys and writes the
//          rows through shared memory as coalesced 16-byte streaming stores.
//          No warp ever waits for another.  The *_count entry points run the
//          count pass without descriptors.  Output order is deterministic:
//          probe order, then R run order.
// The same kernels serve the sort index (runs by binary search) and the left
// outer join (OUTER: a probe without matches yields one NULL-extended row).
#include <climits>

#include "ej_device.cuh"
#include "dir.cuh"
#include "hash_join.cuh"
#include "probe.cuh"
#include "probe_write.cuh"

namespace {


// Row bounds of every bucket of the hash-sorted table (tables planned
// without a key directory): row i (i = nR: the end) begins the buckets between
// the bucket of row i - 1 and its own; each warp takes 256 consecutive rows.
__global__ void __launch_bounds__(256)
bucket_start_kernel(const int32_t* __restrict__ rval, uint64_t nR, uint2* __restrict__ bucket, uint32_t hb) {
  const uint64_t r0 = ((uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5)) * 256;
  if (r0 <= nR) ej_bucket_bounds_warp(rval, nR, r0, hb, bucket, EjHashBucketOf{hb});
}

// ---- key directory of a single table (dir.cuh) -------------------------------

__global__ void __launch_bounds__(DIR_THREADS) dir_count_kernel(const int32_t* __restrict__ rval, uint64_t n,
                                                                uint32_t* __restrict__ tile_keys) {
  const uint32_t total = dir_tile_keys(rval, n, (uint64_t)blockIdx.x * DIR_TILE);
  if (threadIdx.x == 0) tile_keys[blockIdx.x] = total;
}

// per tile: the largest home_k - k; the header (key count, bits, first hash).
// The directory is kept when the table's runs average two rows or more, or
// when the caller expects 16 probes per row or more (prefer_dir): there a
// probe's single slot load repays the build; else the header says bits = 0
// and the table is probed through bucket bounds (dir_bucket_kernel), whose
// build is one launch.
__global__ void __launch_bounds__(DIR_THREADS) dir_tilemax_kernel(const int32_t* __restrict__ rval, uint64_t n,
                                                                  const uint32_t* __restrict__ tile_off,
                                                                  uint32_t ntiles, long long* __restrict__ kmax,
                                                                  DirHeader* hdr, uint32_t prefer_dir) {
  const unsigned long long nk = tile_off[ntiles];
  if (!prefer_dir && 2 * nk > n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      hdr->bits = 0u;
      hdr->nkeys = nk;
    }
    return;
  }
  const uint32_t bits = dir_bits_for(nk, n);
  const long long m = dir_tile_max(rval, n, (uint64_t)blockIdx.x * DIR_TILE, tile_off[blockIdx.x], bits, &hdr->hash0);
  if (threadIdx.x == 0) kmax[blockIdx.x] = m;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hdr->bits = bits;
    hdr->nkeys = nk;
  }
}

// exclusive prefix maximum over the tiles (one block)
__global__ void __launch_bounds__(1024) dir_prefix_kernel(const long long* __restrict__ kmax, uint32_t ntiles,
                                                          long long* __restrict__ kpre,
                                                          const DirHeader* __restrict__ hdr) {
  __shared__ long long tmp[1024 / 32];
  if (hdr->bits == 0) return;  // bucket bounds instead
  const uint64_t per = (ntiles + blockDim.x - 1) / blockDim.x;
  const uint64_t c0 = min((uint64_t)ntiles, threadIdx.x * per), c1 = min((uint64_t)ntiles, c0 + per);
  long long m = LLONG_MIN;
  for (uint64_t c = c0; c < c1; c += 8) {  // eight independent loads in flight
    long long x[8];
#pragma unroll
    for (int u = 0; u < 8; u++) x[u] = c + u < c1 ? kmax[c + u] : LLONG_MIN;
#pragma unroll
    for (int u = 0; u < 8; u++) m = max(m, x[u]);
  }
  long long all;
  long long run = dir_block_exclusive_max(m, tmp, &all);
  for (uint64_t c = c0; c < c1; c += 8) {
    long long x[8];
#pragma unroll
    for (int u = 0; u < 8; u++) x[u] = c + u < c1 ? kmax[c + u] : LLONG_MIN;
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (c + u < c1) {
        kpre[c + u] = run;
        run = max(run, x[u]);
      }
  }
}

__global__ void __launch_bounds__(DIR_THREADS) dir_place_kernel(const int32_t* __restrict__ rval, uint64_t n,
                                                                const uint32_t* __restrict__ tile_off,
                                                                const long long* __restrict__ kpre, DirHeader* hdr,
                                                                uint2* __restrict__ dir, uint32_t packed) {
  if (hdr->bits == 0) return;  // bucket bounds instead
  dir_tile_place(rval, n, (uint64_t)blockIdx.x * DIR_TILE, tile_off[blockIdx.x], kpre[blockIdx.x], hdr, dir,
                 packed != 0);
}

__global__ void __launch_bounds__(256) dir_edge_kernel(const DirHeader* __restrict__ hdr, uint64_t n,
                                                       uint2* __restrict__ dir, uint32_t packed) {
  if (hdr->bits == 0) return;  // bucket bounds instead
  dir_edges(hdr, n, dir, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x,
            packed != 0);
}

// bucket bounds of a table whose header chose them over the directory; a
// few blocks per SM stride over the rows, so that the launch costs next to
// nothing when the directory stays
__global__ void __launch_bounds__(256)
dir_bucket_kernel(const int32_t* __restrict__ rval, uint64_t nR, uint2* __restrict__ bucket, uint32_t hb,
                  const DirHeader* __restrict__ hdr) {
  if (hdr->bits != 0) return;
  const uint64_t warps = (uint64_t)gridDim.x * 8;
  for (uint64_t w = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5); w * 256 <= nR; w += warps)
    ej_bucket_bounds_warp(rval, nR, w * 256, hb, bucket, EjHashBucketOf{hb});
}

// the value buckets of a val-sorted table of n rows (2^hb buckets): the
// smallest and largest vals and the shift that maps their range below 2^hb
__global__ void vbucket_header_kernel(const int32_t* __restrict__ rval, uint64_t n, uint32_t hb,
                                      EjValueBuckets* __restrict__ hdr) {
  EjValueBuckets b = {1, 0, 0u, 0u};  // no rows: an empty range
  if (n) {
    b.vmin = rval[0];
    b.vmax = rval[n - 1];
    const uint32_t range = (uint32_t)b.vmax - (uint32_t)b.vmin;
    const uint32_t len = range ? 32u - (uint32_t)__clz(range) : 0u;
    b.vshift = len > hb ? len - hb : 0u;
  }
  *hdr = b;
}

// bounds of the value buckets: rows [r0, r0 + 256) per warp
__global__ void __launch_bounds__(256)
vbucket_start_kernel(const int32_t* __restrict__ rval, uint64_t nR, uint2* __restrict__ bucket, uint32_t hb,
                     const EjValueBuckets* __restrict__ hdr) {
  const uint64_t r0 = ((uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5)) * 256;
  const EjValueBuckets b = *hdr;
  if (r0 <= nR) ej_bucket_bounds_warp(rval, nR, r0, hb, bucket, EjValueBucketOf{b.vmin, b.vshift});
}

// ---- count, then write from the run descriptors ---------------------------------
// (probe_write.cuh); the warp-tile totals are scanned in between

// L2 prefetch of the 1 KB of one warp tile's probe tuples (or descriptors,
// also 8 bytes per probe), one 128-byte line per lane of the first eight;
// lines past the nP probes are skipped
__device__ __forceinline__ void ej_prefetch_tile(const void* base, uint64_t w, uint64_t nP, unsigned lane) {
  const uint64_t off = w * (PR_WTILE * 8) + (uint64_t)lane * 128u;
  if (lane < 8u && off < nP * 8) asm volatile("prefetch.global.L2 [%0];" ::"l"(static_cast<const char*>(base) + off));
}

// The probe kernels come in two block shapes, WARPS = 8 or 4 warps of one
// 128-probe warp tile each (EJ_OPT_PROBE_WARPS and the tuning table choose).
template <int KIND, bool OUTER, int DESC, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 40 / WARPS)  // 40 warps per SM hide the table loads
probe_count_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t, unsigned long long* __restrict__ wcount,
                   uint64_t nwtiles, void* __restrict__ desc, uint64_t ahead) {
  const uint64_t w = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
  if (w >= nwtiles) return;
  ej_prefetch_tile(P, w + ahead, nP, threadIdx.x & 31u);  // the tile a warp one resident wave later takes
  const unsigned long long total = ej_probe_count_warp_desc<KIND, OUTER, DESC>(P, w * PR_WTILE, nP, t, desc);
  if ((threadIdx.x & 31u) == 0) wcount[w] = total;
}

// Count pass over a packed key directory (inner join, hash table), lean: a
// directory entry {hash, start << 5 | run length} is already the packed run
// descriptor of the write pass (escape 31 included), so a probe costs its
// hash, one 16-byte load of its home pair of slots (more only past smaller
// hashes, or for a run of 31 rows or more) and the store of the entry's
// second word.  Each warp takes two 128-probe tiles, 8 probes per lane
// loaded two at a time (16-byte loads), so that twice the directory loads
// are in flight per warp.  Tiles that are not full (the last warp's) and
// tables whose build chose bucket bounds (bits = 0 in the header) take the
// general path.  STORE: the descriptors are kept for the write pass.
constexpr int PCD_TILES = 2;  // warp tiles per warp

template <bool STORE>
__global__ void __launch_bounds__(256, 4)
probe_count_dir_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t,
                       unsigned long long* __restrict__ wcount, uint64_t nwtiles, uint32_t* __restrict__ desc,
                       uint64_t ahead) {
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t w0 = ((uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5)) * PCD_TILES;
  if (w0 >= nwtiles) return;
  {  // the two tiles a warp one resident wave later takes: 2 KB, lanes 0..15
    const uint64_t off = (w0 + ahead) * (PR_WTILE * 8) + (uint64_t)lane * 128u;
    if (lane < 16u && off < nP * 8) asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char*>(P) + off));
  }
  const uint32_t bits = __ldg(t.dir_bits);
  const uint64_t base = w0 * PR_WTILE;
  if (bits == 0 || base + PCD_TILES * PR_WTILE > nP) {
    for (int k = 0; k < PCD_TILES; k++) {
      const uint64_t w = w0 + k;
      if (w >= nwtiles) break;
      const unsigned long long total =
          STORE ? ej_probe_count_warp_desc<EJ_TABLE_HASH, false, EJ_DESC_PACKED>(P, w * PR_WTILE, nP, t, desc)
                : ej_probe_count_warp_desc<EJ_TABLE_HASH, false, EJ_DESC_NONE>(P, w * PR_WTILE, nP, t, nullptr);
      if (lane == 0) wcount[w] = total;
    }
    return;
  }
  constexpr int N = 4 * PCD_TILES;  // probes per lane
  const uint32_t end = (uint32_t)t.nR << 5;  // entries at or past it: no key (sentinels)
  // probe 2q + e of the lane sits at P[base + 64 q + 2 lane + e]: probes
  // 0..3 in the first tile, 4..7 in the second
  const int4* P4 = reinterpret_cast<const int4*>(P + base) + lane;
  uint32_t hv[N], slot[N];
  bool ok[N], hasb[N];
  uint2 a[N], b[N];
#pragma unroll
  for (int q = 0; q < N / 2; q++) {
    const int4 x = __ldcs(P4 + 32 * q);
    hv[2 * q] = ej_hash32((uint32_t)x.y);
    hv[2 * q + 1] = ej_hash32((uint32_t)x.w);
    ok[2 * q] = ok[2 * q + 1] = true;
  }
  ej_dir_walk<N>(t.dir, 32u - bits, hv, ok, a, b, hasb, slot);
  uint32_t d[N], sum[PCD_TILES] = {};
#pragma unroll
  for (int j = 0; j < N; j++) {
    d[j] = (a[j].x == hv[j] && a[j].y < end) ? a[j].y : 0u;
    uint32_t c = d[j] & 31u;
    if (c == 31u) {  // 31 rows or more: the next slot starts the next run
      const uint32_t start = d[j] >> 5;
      uint32_t next = (hasb[j] ? b[j] : __ldg(t.dir + slot[j] + 1)).y >> 5;
      while (next == start) next = __ldg(t.dir + ++slot[j] + 1).y >> 5;  // a guard
      c = next - start;
    }
    sum[j / 4] += c;  // a lane's runs: under 4 x 2^27 rows per tile
  }
  if (STORE) {
    uint2* D2 = reinterpret_cast<uint2*>(desc + base) + lane;
#pragma unroll
    for (int q = 0; q < N / 2; q++) __stcs(D2 + 32 * q, make_uint2(d[2 * q], d[2 * q + 1]));
  }
#pragma unroll
  for (int k = 0; k < PCD_TILES; k++) {
    // the tile's rows (under 2^34): 32-bit sums of the lanes' 16-bit halves
    const uint32_t lo16 = __reduce_add_sync(EJ_FULL_MASK, sum[k] & 0xFFFFu);
    const uint32_t hi16 = __reduce_add_sync(EJ_FULL_MASK, sum[k] >> 16);
    if (lane == 0) wcount[w0 + k] = ((unsigned long long)hi16 << 16) + lo16;
  }
}

template <int KIND, bool OUTER, int DESC, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
probe_write_kernel(const ej_tuple* __restrict__ P, const void* __restrict__ desc, uint64_t nP, ej_table_view t,
                   const unsigned long long* __restrict__ woff, uint64_t nwtiles, ej_result* __restrict__ out,
                   uint64_t cap, ej_dev_status* st, uint64_t ahead) {
  __shared__ int4 stage[WARPS][PW_STAGE_ROWS];
  const unsigned int warp = threadIdx.x >> 5;
  const uint64_t w = (uint64_t)blockIdx.x * WARPS + warp;
  if (w >= nwtiles) return;
  if (w == 0 && threadIdx.x == 0 && woff[nwtiles] > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
  ej_prefetch_tile(P, w + ahead, nP, threadIdx.x & 31u);  // the tile a warp one resident wave later takes
  // the tile's descriptors: 1 KB (wide, lanes 8..15) or 512 bytes (packed, lanes 8..11)
  if (DESC == EJ_DESC_NONE) {
  } else if (DESC == EJ_DESC_PACKED) {
    const unsigned l = (threadIdx.x & 31u) - 8u;
    const uint64_t doff = (w + ahead) * (PR_WTILE * 4) + (uint64_t)l * 128u;
    if (l < 4u && doff < nP * 4) asm volatile("prefetch.global.L2 [%0];" ::"l"(static_cast<const char*>(desc) + doff));
  } else {
    ej_prefetch_tile(desc, w + ahead, nP, (threadIdx.x & 31u) - 8u);
  }
  const unsigned long long off = woff[w];
  if (off >= cap) return;
  ej_probe_write_warp<KIND, OUTER, DESC>(P, desc, w * PR_WTILE, nP, t, off, out, cap, stage[warp]);
}

// One pass (the joins that materialise rows in one call): each warp finds the
// runs of its 128 probes, reserves its rows with one atomic add on the row
// cursor, and writes them through its staging buffer as the write pass does.
// Warps take their row ranges in the order they reach the cursor, so the row
// order is not deterministic (the multiset is); rows at or past cap are
// dropped, the cursor ends at the exact count.  KEYS: how the run keys are
// loaded (ej_probe_prefetch), fixed per table by the host.
template <int KIND, bool OUTER, int KEYS, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
probe_fused_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t, uint64_t nwtiles,
                   unsigned long long* __restrict__ cursor, ej_result* __restrict__ out, uint64_t cap,
                   ej_dev_status* st, uint64_t ahead) {
  __shared__ int4 stage[WARPS][PW_STAGE_ROWS];
  const unsigned int warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint64_t w = (uint64_t)blockIdx.x * WARPS + warp;
  if (w >= nwtiles) return;
  ej_prefetch_tile(P, w + ahead, nP, lane);  // the tile a warp one resident wave later takes
  EjProbeWarp pw;
  ej_probe_runs_warp<KIND, OUTER>(P, w * PR_WTILE, nP, t, pw);
  unsigned long long mine = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) mine += pw.cnt[j];
  const unsigned long long total = ej_warp_sum<unsigned long long>(mine);
  if (total == 0) return;
  // the run keys and the row reservation travel together: the key loads are
  // issued first and do not wait for the atomic's answer
  int32_t kk[PR_ITEMS][PW_PREFETCH];
  ej_probe_prefetch<KEYS>(t, pw, kk);
  unsigned long long off = 0;
  if (lane == 0) {
    off = atomicAdd(cursor, total);
    if (off + total > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
  }
  off = __shfl_sync(EJ_FULL_MASK, off, 0);
  if (off >= cap) return;
  ej_emit_warp(pw, kk, t, off, out, cap, stage[warp]);
}

// the descriptor form of a table: packed (4 bytes) when its row positions fit
// in 27 bits, else wide; the count and the write pass of one probe decide it
// from the same table view
static int desc_form(const ej_table_view& t) { return t.nR < EJ_PACKED_MAX_ROWS ? EJ_DESC_PACKED : EJ_DESC_WIDE; }

template <int KIND, bool OUTER, int WARPS>
ej_status launch_count_w(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         unsigned long long* wcount, void* desc) {
  const uint64_t ahead = (uint64_t)h->num_sms * 40;  // warp tiles of one resident wave
  const dim3 grid((unsigned)pp.ntiles);
  constexpr int TH = WARPS * 32;
  // inner probes of a packed key directory, 16-byte aligned: the lean count
  // (8 warps of two tiles per block, 4 blocks per SM)
  if (KIND == EJ_TABLE_HASH && !OUTER && t.dir && t.dir_packed && (reinterpret_cast<uintptr_t>(P) & 15u) == 0 &&
      (!desc || desc_form(t) == EJ_DESC_PACKED)) {
    const uint64_t blocks = (pp.nwtiles + 8 * PCD_TILES - 1) / (8 * PCD_TILES);
    const uint64_t ahead2 = (uint64_t)h->num_sms * 4 * 8 * PCD_TILES;  // warp tiles of one resident wave
    if (desc)
      probe_count_dir_kernel<true><<<(unsigned)blocks, 256, 0, h->stream>>>(
          P, pp.nP, t, wcount, pp.nwtiles, static_cast<uint32_t*>(desc), ahead2);
    else
      probe_count_dir_kernel<false><<<(unsigned)blocks, 256, 0, h->stream>>>(P, pp.nP, t, wcount, pp.nwtiles,
                                                                              nullptr, ahead2);
    return ej_check_launch(h, "probe_count_dir_kernel");
  }
  if (!desc || desc_form(t) == EJ_DESC_NONE)
    probe_count_kernel<KIND, OUTER, EJ_DESC_NONE, WARPS><<<grid, TH, 0, h->stream>>>(P, pp.nP, t, wcount, pp.nwtiles,
                                                                                     nullptr, ahead);
  else if (desc_form(t) == EJ_DESC_PACKED)
    probe_count_kernel<KIND, OUTER, EJ_DESC_PACKED, WARPS><<<grid, TH, 0, h->stream>>>(P, pp.nP, t, wcount,
                                                                                       pp.nwtiles, desc, ahead);
  else
    probe_count_kernel<KIND, OUTER, EJ_DESC_WIDE, WARPS><<<grid, TH, 0, h->stream>>>(P, pp.nP, t, wcount, pp.nwtiles,
                                                                                     desc, ahead);
  return ej_check_launch(h, "probe_count_kernel");
}

template <int KIND, bool OUTER>
ej_status launch_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       unsigned long long* wcount, void* desc) {
  return pp.warps == 4 ? launch_count_w<KIND, OUTER, 4>(h, pp, P, t, wcount, desc)
                       : launch_count_w<KIND, OUTER, 8>(h, pp, P, t, wcount, desc);
}

template <int KIND, bool OUTER, int WARPS>
ej_status launch_write_w(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         const void* desc, const unsigned long long* woff, ej_result* out, uint64_t cap) {
  const uint64_t ahead = (uint64_t)h->num_sms * 32;  // warp tiles of one resident wave
  const dim3 grid((unsigned)pp.ntiles);
  constexpr int TH = WARPS * 32;
  if (desc_form(t) == EJ_DESC_NONE)
    probe_write_kernel<KIND, OUTER, EJ_DESC_NONE, WARPS><<<grid, TH, 0, h->stream>>>(
        P, nullptr, pp.nP, t, woff, pp.nwtiles, out, cap, h->d_status, ahead);
  else if (desc_form(t) == EJ_DESC_PACKED)
    probe_write_kernel<KIND, OUTER, EJ_DESC_PACKED, WARPS><<<grid, TH, 0, h->stream>>>(
        P, desc, pp.nP, t, woff, pp.nwtiles, out, cap, h->d_status, ahead);
  else
    probe_write_kernel<KIND, OUTER, EJ_DESC_WIDE, WARPS><<<grid, TH, 0, h->stream>>>(
        P, desc, pp.nP, t, woff, pp.nwtiles, out, cap, h->d_status, ahead);
  return ej_check_launch(h, "probe_write_kernel");
}

template <int KIND, bool OUTER>
ej_status launch_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       const void* desc, const unsigned long long* woff, ej_result* out, uint64_t cap) {
  return pp.warps == 4 ? launch_write_w<KIND, OUTER, 4>(h, pp, P, t, desc, woff, out, cap)
                       : launch_write_w<KIND, OUTER, 8>(h, pp, P, t, desc, woff, out, cap);
}

}  // namespace

uint32_t ej_table_bucket_bits(uint64_t nR, int delta) {
  const int lg = (int)ej_ceil_log2(nR < 2 ? 2 : nR);
  int hb = lg - 2 + delta;  // about four R tuples per bucket at delta 0
  if (hb < 1) hb = 1;
  if (hb > 30) hb = 30;
  return (uint32_t)hb;
}

// ---- table build --------------------------------------------------------


size_t ej_table_aux_bytes(const ej_table_plan_t& tp) {
  const size_t buckets = (size_t(1) << tp.hb) * sizeof(uint2);
  if (tp.kind != EJ_TABLE_HASH) return EJ_VBUCKET_HEADER_BYTES + buckets;
  // a directory table keeps room for the bucket bounds its build may choose instead
  return tp.use_dir ? DIR_HEADER_BYTES + ej_dir_capacity(tp.nR) * sizeof(uint2) + buckets : buckets;
}

size_t ej_table_col_bytes(uint64_t nR) { return (size_t)(nR + EJ_TABLE_PAD) * sizeof(int32_t); }

ej_table_knobs ej_tuned_table_knobs(const ej_handle* h, uint64_t nR) {
  ej_table_knobs k;
  k.delta = ej_tuned_bucket_delta(h, nR);
  k.build = ej_tuned_build(h, nR);
  k.table = ej_tuned_table_format(h, nR);
  return k;
}

void ej_table_plan(ej_plan_bytes& p, ej_table_plan_t& tp, uint64_t nR, bool own_storage, int kind,
                   const ej_table_knobs& k, uint64_t n_probe) {
  tp.kind = kind;
  tp.nR = nR;
  // a directory chosen by the tuning is kept whatever the runs' length
  tp.prefer_dir = n_probe > 16 * nR || k.table == EJ_TABLE_FORMAT_DIRECTORY;
  tp.use_dir = kind == EJ_TABLE_HASH &&
               (k.table == EJ_TABLE_FORMAT_DIRECTORY ||
                (k.table == EJ_TABLE_FORMAT_PLANNER &&
                 (nR >= EJ_DIR_MIN_ROWS || (tp.prefer_dir && nR >= EJ_DIR_PROBE_MIN_ROWS))));
  tp.hb = ej_table_bucket_bits(nR, k.delta);  // hash buckets, or value buckets of a sorted table
  tp.passes = 4;  // all 32 key bits: equal keys end up adjacent
  if (!own_storage) {
    tp.rkey_off = p.add(ej_table_col_bytes(nR));
    tp.rval_off = p.add(ej_table_col_bytes(nR));
    tp.aux_off = p.add(ej_table_aux_bytes(tp));
  }
  const size_t tuples = (size_t)(nR ? nR : 1) * sizeof(ej_tuple);
  tp.tmp_a_off = p.add(tuples);
  tp.tmp_b_off = p.add(tuples);
  tp.msd = kind == EJ_TABLE_HASH &&
           (k.build == EJ_BUILD_MSD || (k.build == EJ_BUILD_PLANNER && nR >= EJ_MSD_MIN_ROWS));
  // onesweep only when chosen: its per-digit look-back measured slower than
  // the three-launch LSD pass at every size (sort index of 2^24 rows: 0.68 vs
  // 0.58 ms)
  tp.onesweep = !tp.msd && k.build == EJ_BUILD_ONESWEEP;
  if (tp.msd)
    ej_msd_plan_add(p, tp.mplan, nR);
  else if (tp.onesweep)
    ej_onesweep_plan_add(p, tp.oplan, nR);
  else
    ej_radix_plan_add(p, tp.rplan, nR);
  if (tp.use_dir) {  // directory build scratch
    const uint64_t tiles = (nR + DIR_TILE - 1) / DIR_TILE + 1;
    tp.dir_keys_off = p.add(tiles * sizeof(uint32_t));
    tp.dir_off_off = p.add((tiles + 1) * sizeof(uint32_t));
    tp.dir_scan_off = p.add(ej_scan_scratch_bytes(tiles));
    tp.dir_kmax_off = p.add(tiles * sizeof(long long));
    tp.dir_kpre_off = p.add(tiles * sizeof(long long));
  }
}

size_t ej_table_bytes(uint64_t nR, int delta) {
  const uint32_t hb = ej_table_bucket_bits(nR, delta);
  return (size_t)nR * sizeof(ej_tuple) + (size_t(1) << hb) * sizeof(uint2);
}

ej_status ej_table_build(ej_handle* h, const ej_table_plan_t& tp, const ej_tuple* R, int32_t* rkey, int32_t* rval,
                         void* aux, ej_table_view* view) {
  // LSD passes over the 32-bit key (hash32(val), or the order-preserving image
  // of val for a sorted index), least significant byte first; the last pass
  // writes the two columns
  const int digit_kind = tp.kind == EJ_TABLE_HASH ? EJ_DIGIT_HASH : EJ_DIGIT_VALUE;
  ej_tuple* tmp[2] = {reinterpret_cast<ej_tuple*>(ej_arena_at(h, tp.tmp_a_off)),
                      reinterpret_cast<ej_tuple*>(ej_arena_at(h, tp.tmp_b_off))};
  const ej_tuple* src = R;
  if (tp.msd) EJ_TRY(ej_msd_sort(h, tp.mplan, R, tmp[0], tmp[1], rkey, rval));
  if (tp.onesweep) EJ_TRY(ej_onesweep_sort(h, tp.oplan, R, tmp[0], tmp[1], rkey, rval, digit_kind));
  for (uint32_t p = 0; p < tp.passes && tp.nR && !tp.msd && !tp.onesweep; p++) {
    const uint32_t shift = 8u * p;
    if (p + 1 == tp.passes) {
      EJ_TRY(ej_radix_pass_soa(h, tp.rplan, src, rkey, rval, shift, 8u, digit_kind));
    } else {
      if (p == 0)
        EJ_TRY(ej_partition_pass(h, tp.rplan, src, tmp[0], shift, 8u, digit_kind));
      else
        EJ_TRY(ej_radix_pass(h, tp.rplan, src, tmp[p & 1], shift, 8u, digit_kind));
      src = tmp[p & 1];
    }
  }
  view->kind = tp.kind;
  view->rkey = rkey;
  view->rval = rval;
  view->nR = tp.nR;
  view->hb = tp.hb;
  if (tp.kind == EJ_TABLE_HASH && !tp.use_dir) {
    uint2* bucket = static_cast<uint2*>(aux);
    const uint64_t blocks = (tp.nR + 1 + 2047) / 2048;  // 256 rows per warp, 8 warps per block
    bucket_start_kernel<<<(unsigned)blocks, 256, 0, h->stream>>>(rval, tp.nR, bucket, tp.hb);
    EJ_TRY(ej_check_launch(h, "bucket_start_kernel"));
    view->bucket = bucket;
  } else if (tp.kind == EJ_TABLE_HASH) {
    DirHeader* hdr = static_cast<DirHeader*>(aux);
    uint2* dir = reinterpret_cast<uint2*>(static_cast<char*>(aux) + DIR_HEADER_BYTES);
    uint2* bucket = dir + ej_dir_capacity(tp.nR);
    const uint32_t tiles = (uint32_t)((tp.nR + DIR_TILE - 1) / DIR_TILE);
    uint32_t* keys = reinterpret_cast<uint32_t*>(ej_arena_at(h, tp.dir_keys_off));
    uint32_t* off = reinterpret_cast<uint32_t*>(ej_arena_at(h, tp.dir_off_off));
    long long* kmax = reinterpret_cast<long long*>(ej_arena_at(h, tp.dir_kmax_off));
    long long* kpre = reinterpret_cast<long long*>(ej_arena_at(h, tp.dir_kpre_off));
    const uint32_t packed = tp.nR < (1ull << 27) ? 1u : 0u;  // start << 5 | run length fits 32 bits
    if (tiles) {
      dir_count_kernel<<<tiles, 256, 0, h->stream>>>(rval, tp.nR, keys);
      EJ_TRY(ej_check_launch(h, "dir_count_kernel"));
      EJ_TRY(ej_scan_u32_u32(h, keys, tiles, off, ej_arena_at(h, tp.dir_scan_off)));
      dir_tilemax_kernel<<<tiles, 256, 0, h->stream>>>(rval, tp.nR, off, tiles, kmax, hdr, tp.prefer_dir ? 1u : 0u);
      EJ_TRY(ej_check_launch(h, "dir_tilemax_kernel"));
      dir_prefix_kernel<<<1, 1024, 0, h->stream>>>(kmax, tiles, kpre, hdr);
      EJ_TRY(ej_check_launch(h, "dir_prefix_kernel"));
      dir_place_kernel<<<tiles, 256, 0, h->stream>>>(rval, tp.nR, off, kpre, hdr, dir, packed);
      EJ_TRY(ej_check_launch(h, "dir_place_kernel"));
      const uint64_t bblocks = std::min<uint64_t>((tp.nR + 1 + 2047) / 2048, (uint64_t)h->num_sms * 8);
      dir_bucket_kernel<<<(unsigned)bblocks, 256, 0, h->stream>>>(rval, tp.nR, bucket, tp.hb, hdr);
      EJ_TRY(ej_check_launch(h, "dir_bucket_kernel"));
    } else {  // no rows: no keys, two home slots
      const DirHeader empty = {1u, 0u, 0ull, 0ull, 0ull, 0u, 0u};
      EJ_CUDA(h, cudaMemcpyAsync(hdr, &empty, sizeof empty, cudaMemcpyHostToDevice, h->stream));
    }
    dir_edge_kernel<<<(unsigned)h->num_sms * 4, 256, 0, h->stream>>>(hdr, tp.nR, dir, packed);
    EJ_TRY(ej_check_launch(h, "dir_edge_kernel"));
    view->dir = dir;
    view->dir_bits = &hdr->bits;
    view->dir_packed = packed;
    view->bucket = bucket;
  } else {  // sorted: value buckets, header first
    EjValueBuckets* vh = static_cast<EjValueBuckets*>(aux);
    uint2* bucket = reinterpret_cast<uint2*>(static_cast<char*>(aux) + EJ_VBUCKET_HEADER_BYTES);
    vbucket_header_kernel<<<1, 1, 0, h->stream>>>(rval, tp.nR, tp.hb, vh);
    EJ_TRY(ej_check_launch(h, "vbucket_header_kernel"));
    const uint64_t blocks = (tp.nR + 1 + 2047) / 2048;  // 256 rows per warp, 8 warps per block
    vbucket_start_kernel<<<(unsigned)blocks, 256, 0, h->stream>>>(rval, tp.nR, bucket, tp.hb, vh);
    EJ_TRY(ej_check_launch(h, "vbucket_start_kernel"));
    view->bucket = bucket;
    view->vbuckets = vh;
  }
  return EJ_OK;
}

// ---- probe --------------------------------------------------------------

void ej_probe_plan(ej_plan_bytes& p, ej_probe_plan_t& pp, uint64_t nP, bool with_desc, uint32_t warps) {
  pp.nP = nP;
  pp.warps = warps == 4 ? 4u : 8u;
  pp.nwtiles = (nP + PR_WTILE - 1) / PR_WTILE;
  pp.ntiles = (pp.nwtiles + pp.warps - 1) / pp.warps;
  pp.count_off = p.add((pp.nwtiles + 1) * sizeof(unsigned long long));
  pp.off_off = p.add((pp.nwtiles + 1) * sizeof(unsigned long long));
  pp.scan_off = p.add(ej_scan_scratch_bytes(pp.nwtiles));
  pp.with_desc = with_desc;
  if (with_desc) pp.desc_off = p.add((size_t)(nP ? nP : 1) * sizeof(uint2));
}

ej_status ej_probe_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, unsigned long long* d_count) {
  unsigned long long* wcount = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.count_off));
  unsigned long long* woff = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.off_off));
  void* desc = pp.with_desc ? ej_arena_at(h, pp.desc_off) : nullptr;
  if (pp.ntiles) {
    if (t.kind == EJ_TABLE_HASH)
      EJ_TRY(outer ? launch_count<EJ_TABLE_HASH, true>(h, pp, P, t, wcount, desc)
                   : launch_count<EJ_TABLE_HASH, false>(h, pp, P, t, wcount, desc));
    else
      EJ_TRY(outer ? launch_count<EJ_TABLE_SORTED, true>(h, pp, P, t, wcount, desc)
                   : launch_count<EJ_TABLE_SORTED, false>(h, pp, P, t, wcount, desc));
  }
  EJ_TRY(ej_scan_u64_u64(h, wcount, pp.nwtiles, woff, ej_arena_at(h, pp.scan_off)));
  if (d_count)
    EJ_CUDA(h, cudaMemcpyAsync(d_count, woff + pp.nwtiles, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                               h->stream));
  return EJ_OK;
}

ej_status ej_probe_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         ej_result* out, uint64_t cap, bool outer) {
  if (!pp.ntiles) return EJ_OK;
  if (!pp.with_desc) return ej_fail(h, EJ_ERR_INTERNAL, "probe write planned without run descriptors");
  const void* desc = ej_arena_at(h, pp.desc_off);
  const unsigned long long* woff = reinterpret_cast<const unsigned long long*>(ej_arena_at(h, pp.off_off));
  if (t.kind == EJ_TABLE_HASH)
    return outer ? launch_write<EJ_TABLE_HASH, true>(h, pp, P, t, desc, woff, out, cap)
                 : launch_write<EJ_TABLE_HASH, false>(h, pp, P, t, desc, woff, out, cap);
  return outer ? launch_write<EJ_TABLE_SORTED, true>(h, pp, P, t, desc, woff, out, cap)
               : launch_write<EJ_TABLE_SORTED, false>(h, pp, P, t, desc, woff, out, cap);
}

// ---- partition bits for the probe side ------------------------------------

uint32_t ej_probe_partition_bits(const ej_handle* h, uint64_t nR, uint64_t nS) {
  (void)nS;
  const uint32_t hb = ej_table_bucket_bits(nR, ej_tuned_bucket_delta(h, nR));
  const int forced = ej_tuned_partition_bits(h, nR);
  if (forced >= 0) return std::min<uint32_t>((uint32_t)forced, std::min(hb, 8u));
  const double table = (double)ej_table_bytes(nR, ej_tuned_bucket_delta(h, nR));
  const double l2 = (double)(h->l2_bytes ? h->l2_bytes : (size_t)126 << 20);
  if (table <= l2 / 4.0) return 0;  // the whole table stays L2-resident
  // one partition's table region should be several MB so that the partitions
  // in flight share L2 with the streaming probe and output traffic (C3's
  // 2^26-row tables: 6 bits, a region of L2/8 by the rows and buckets; with
  // the key directory of a quarter load the count's region is 8 MB: the
  // step 21.80 ms at 7 bits, 21.57 at 6)
  uint32_t pb = ej_ceil_log2((uint64_t)(table / (l2 / 8.0)) + 1);
  if (pb > 8) pb = 8;
  if (pb > hb) pb = hb;
  return pb;
}

// ---- probe drivers -------------------------------------------------------

void ej_probe_layout_add(ej_plan_bytes& p, ej_probe_layout& L, uint64_t nS, uint32_t pb, bool count_only,
                         bool two_pass, uint32_t warps) {
  L.pb = pb;
  if (pb) {
    L.spart_off = p.add((size_t)nS * sizeof(ej_tuple));
    ej_radix_plan_add(p, L.splan, nS);
  }
  (void)count_only;
  ej_probe_plan(p, L.pp, nS, two_pass, warps);
}

template <int KIND, bool OUTER, int WARPS>
static ej_status launch_fused_w(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                                unsigned long long* cursor, ej_result* out, uint64_t cap) {
  const uint64_t ahead = (uint64_t)h->num_sms * 32;  // warp tiles of one resident wave
  if (t.short_runs)
    probe_fused_kernel<KIND, OUTER, EJ_KEYS_CHUNKS, WARPS><<<(unsigned)pp.ntiles, WARPS * 32, 0, h->stream>>>(
        P, pp.nP, t, pp.nwtiles, cursor, out, cap, h->d_status, ahead);
  else
    probe_fused_kernel<KIND, OUTER, EJ_KEYS_WINDOW, WARPS><<<(unsigned)pp.ntiles, WARPS * 32, 0, h->stream>>>(
        P, pp.nP, t, pp.nwtiles, cursor, out, cap, h->d_status, ahead);
  return ej_check_launch(h, "probe_fused_kernel");
}

template <int KIND, bool OUTER>
static ej_status launch_fused(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                              unsigned long long* cursor, ej_result* out, uint64_t cap) {
  return pp.warps == 4 ? launch_fused_w<KIND, OUTER, 4>(h, pp, P, t, cursor, out, cap)
                       : launch_fused_w<KIND, OUTER, 8>(h, pp, P, t, cursor, out, cap);
}

// [partition +] the fused pass; the count ends in *cursor (zeroed here)
static ej_status ej_probe_fused(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                                bool outer, ej_result* out, uint64_t cap, unsigned long long* cursor) {
  EJ_CUDA(h, cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), h->stream));
  if (!pp.ntiles) return EJ_OK;
  if (t.kind == EJ_TABLE_HASH)
    return outer ? launch_fused<EJ_TABLE_HASH, true>(h, pp, P, t, cursor, out, cap)
                 : launch_fused<EJ_TABLE_HASH, false>(h, pp, P, t, cursor, out, cap);
  return outer ? launch_fused<EJ_TABLE_SORTED, true>(h, pp, P, t, cursor, out, cap)
               : launch_fused<EJ_TABLE_SORTED, false>(h, pp, P, t, cursor, out, cap);
}

// Partition S (when the layout says so), count (+ scan), then write unless
// counting only; records phase marks 2..4 (the caller has begun the set and
// marked the build).  The arena must already hold the layout, reserved
// together with anything the table placed there, so that no reservation
// moves a built table.
ej_status ej_probe_exec(ej_handle* h, const ej_probe_layout& L, const ej_table_view& t, const ej_tuple* S,
                        bool outer, bool count_only, ej_result* out, uint64_t out_cap,
                        unsigned long long* d_count) {
  const ej_tuple* P = S;
  if (L.pb) {
    ej_tuple* spart = reinterpret_cast<ej_tuple*>(ej_arena_at(h, L.spart_off));
    EJ_TRY(ej_partition_pass(h, L.splan, S, spart, 32u - L.pb, L.pb));
    P = spart;
  }
  ej_phase_mark(h, 2);
  if (count_only || L.pp.with_desc) {  // the count pass, then (planned two-pass) rows in probe order
    EJ_TRY(ej_probe_count(h, L.pp, P, t, outer, d_count));
    ej_phase_mark(h, 3);
    if (!count_only) EJ_TRY(ej_probe_write(h, L.pp, P, t, out, out_cap, outer));
  } else {
    ej_phase_mark(h, 3);  // one pass: recorded as the write phase
    EJ_TRY(ej_probe_fused(h, L.pp, P, t, outer, out, out_cap, d_count ? d_count : h->d_words + 3));
  }
  ej_phase_mark(h, 4);
  return EJ_OK;
}

// the rows of the join whose count the handle kept: the write pass alone,
// from the count's run descriptors and warp-tile offsets
static ej_status hash_join_write_kept(ej_handle* h, ej_result* out, uint64_t out_cap, unsigned long long* d_count) {
  const ej_prepared_join& pj = *h->prep;
  ej_phase_begin(h);
  for (int k = 1; k <= 3; k++) ej_phase_mark(h, k);  // build, partition and count were the count's
  EJ_TRY(ej_probe_write(h, pj.L.pp, pj.P, pj.t, out, out_cap));
  const unsigned long long* woff = reinterpret_cast<const unsigned long long*>(ej_arena_at(h, pj.L.pp.off_off));
  if (d_count)
    EJ_CUDA(h, cudaMemcpyAsync(d_count, woff + pj.L.pp.nwtiles, sizeof(unsigned long long),
                               cudaMemcpyDeviceToDevice, h->stream));
  ej_phase_mark(h, 4);
  // kept for another write only when this one was cut short by the capacity
  h->prep_valid = pj.count_known && out_cap < pj.count;
  return EJ_OK;
}

ej_status ej_hash_join_run(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                           ej_result* out, uint64_t out_cap, unsigned long long* d_count, int mode) {
  // mode: 0 = partition S when the planner says so, 1 = never partition S, 2 = count only
  if (mode == 0 && h->prep_valid && h->prep && h->prep->arena == h->arena && h->prep->R == R &&
      h->prep->nR == nR && h->prep->S == S && h->prep->nS == nS)
    return hash_join_write_kept(h, out, out_cap, d_count);
  // a count keeps its table, partitioned S and run descriptors for the write
  // that follows it
  const bool keep = mode == 2 && h->opt_count_reuse;
  const uint32_t pb = (mode == 1) ? 0u : ej_probe_partition_bits(h, nR, nS);
  ej_plan_bytes p;
  ej_table_plan_t tp;
  ej_table_plan(p, tp, nR, /*own_storage=*/false, EJ_TABLE_HASH, ej_tuned_table_knobs(h, nR), nS);
  ej_probe_layout L;
  // the build-side-only join keeps its rows in probe order (the batched joins
  // give the same rows in the same order); the others take the one-pass probe
  ej_probe_layout_add(p, L, nS, pb, mode == 2, /*two_pass=*/mode == 1 || keep, ej_tuned_probe_warps(h, nR));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_table_view t;
  EJ_TRY(ej_table_build(h, tp, R, reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rkey_off)),
                        reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rval_off)), ej_arena_at(h, tp.aux_off), &t));
  ej_phase_mark(h, 1);
  EJ_TRY(ej_probe_exec(h, L, t, S, /*outer=*/false, mode == 2, out, out_cap, d_count));
  if (keep) {
    if (!h->prep) h->prep = new ej_prepared_join();
    ej_prepared_join& pj = *h->prep;
    pj.R = R;
    pj.nR = nR;
    pj.S = S;
    pj.nS = nS;
    pj.arena = h->arena;
    pj.P = L.pb ? reinterpret_cast<const ej_tuple*>(ej_arena_at(h, L.spart_off)) : S;
    pj.L = L;
    pj.t = t;
    pj.count_known = false;
    h->prep_valid = true;
  }
  return EJ_OK;
}
