// batch.cu - many hash joins as one pipeline.
//
// The reference runs one join per process, every phase its own launch with a
// host synchronisation after it (joins/hashJoin_gpu/main_street/hj.cc:454-475).
// For a stream of joins of uneven sizes (most of them small) that is launch-
// and latency-bound.  Here a batch of joins is one fixed sequence of launches,
// whatever the number of joins in it:
//   build       four segmented LSD radix passes over the joins that are not
//               small: tiles never cross a join and
//               the digit histograms are laid out join by join, so one scan
//               places every join's rows in its own range, hash-sorted (the
//               first pass reads every join's R where it lies)
//   starts      every join's bucket starts in one launch (its own bucket bits;
//               a batch's tables are small enough for L2, where the bucket
//               scan is as fast as a key directory and one launch builds it)
//   probe       one launch over a task list, a task per block: whole small
//               joins (R of at most 2048 rows: table built and probed in
//               shared memory by one CTA, no radix pass) and the probe tiles
//               of the others (each warp finds its runs, reserves its rows
//               with one atomic add on its join's count and writes them, as
//               the one-pass probe of single joins does).
// Every join's rows are the rows it gives alone; their order within the join
// is not specified (warps reserve their ranges in the order they arrive).
#include "ej_device.cuh"
#include "ej_entry.h"
#include "hash_join.cuh"
#include "probe_write.cuh"

namespace {

constexpr uint32_t BX_RX_TILE = EJ_RX_TILE;
static_assert(BX_RX_TILE % 256 == 0, "bucket bounds take 256-row warp spans that must not cross an R tile");

// per join, on the device
struct BatchJoin {
  ej_table_view view;
  const ej_tuple* S;
  ej_result* out;
  unsigned long long cap;
  unsigned long long* d_count;  // the join's row cursor, then its count
  unsigned long long nS;
  unsigned long long nwtiles;  // warp tiles of the join
  unsigned long long r_row0;   // first row of the join in the concatenated R
  const ej_tuple* R;
};

// a task of the batch's task list: one probe tile of a join (local = the
// tile), or a whole small join (local = BX_SMALL_TASK)
struct BatchTask {
  uint32_t join, local;
};
constexpr uint32_t BX_SMALL_TASK = 0xFFFFFFFFu;
// joins of at most this many R rows are built and probed in shared memory
constexpr uint32_t BX_SMALL_R = 2048;
// the planner's load of a batch's bucket bounds, about 2 rows a bucket (its
// probe, bound by the latency of its loads, finds empty buckets without the
// scan; the served stream's 256-instance batch 12.3 -> 11.9 ms against 4
// rows a bucket, 12.3 ms at 1): explicit options and the tuning table first
constexpr int BX_BUCKET_DELTA = 1;

// bucket bounds of every join: the block of one R tile fills the gaps
// between the buckets of consecutive rows of its join; the join's last row
// also fills the tail up to 2^hb
__global__ void batch_bucket_start_kernel(const ej_rx_tile* __restrict__ tiles, const BatchJoin* __restrict__ joins,
                                          uint2* __restrict__ bucket_all, const unsigned long long* bucket_base) {
  const ej_rx_tile d = tiles[blockIdx.x];
  const BatchJoin& j = joins[d.pad];
  const ej_table_view& t = j.view;
  uint2* bucket = bucket_all + bucket_base[d.pad];
  const uint64_t first = d.start - j.r_row0;  // local row index of the tile's first row
  // the join's last tile also takes the end row (local row nR)
  const uint64_t end = first + d.n + (first + d.n == t.nR ? 1u : 0u);
  // tiles are multiples of 256 rows except a join's last, so a warp's 256
  // rows never reach into the next tile
  for (uint64_t r0 = first + (threadIdx.x >> 5) * 256; r0 < end; r0 += (blockDim.x >> 5) * 256)
    ej_bucket_bounds_warp(t.rval, t.nR, r0, t.hb, bucket, EjHashBucketOf{t.hb});
}

// one probe tile of a join whose table the segmented passes built: each warp
// reserves its rows on its join's cursor (d_count, zeroed before the launch),
// so the cursor ends at the join's count
__device__ __forceinline__ void batch_probe_tile(const BatchJoin& j, uint32_t local, int4 (*stage)[PW_STAGE_ROWS],
                                                 ej_dev_status* st) {
  const unsigned int warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint64_t w = (uint64_t)local * PR_WARPS + warp;
  if (w >= j.nwtiles) return;
  EjProbeWarp pw;
  ej_probe_runs_warp<EJ_TABLE_HASH, false>(j.S, w * PR_WTILE, j.nS, j.view, pw);
  unsigned long long mine = 0;
#pragma unroll
  for (int q = 0; q < PR_ITEMS; q++) mine += pw.cnt[q];
  const unsigned long long total = ej_warp_sum<unsigned long long>(mine);
  if (total == 0) return;
  int32_t kk[PR_ITEMS][PW_PREFETCH];
  ej_probe_prefetch<EJ_KEYS_CHUNKS>(j.view, pw, kk);
  unsigned long long off = 0;
  if (lane == 0) {
    off = atomicAdd(j.d_count, total);
    if (off + total > j.cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
  }
  off = __shfl_sync(EJ_FULL_MASK, off, 0);
  if (off >= j.cap) return;
  ej_emit_warp(pw, kk, j.view, off, j.out, j.cap, stage[warp]);
}

// A join small enough for shared memory (nR <= BX_SMALL_R), whole, by one
// CTA: R into a chained hash table in shared memory (bucket heads and row
// links), then S probed 32 rows per warp and round: every lane walks its
// row's chain twice, first counting, then - after one atomic add on the
// join's cursor has reserved the warp's rows - writing them.  No radix pass,
// no table in global memory.
__device__ __forceinline__ void batch_small_join(const BatchJoin& j, int4* smem, ej_dev_status* st) {
  int32_t* rk = reinterpret_cast<int32_t*>(smem);
  int32_t* rv = rk + BX_SMALL_R;
  int32_t* nxt = rv + BX_SMALL_R;
  int32_t* head = nxt + BX_SMALL_R;
  const uint32_t nR = (uint32_t)j.view.nR;
  uint32_t nb = 1;
  while (nb < nR) nb <<= 1;
  for (uint32_t b = threadIdx.x; b < nb; b += PR_THREADS) head[b] = -1;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nR; i += PR_THREADS) {
    const int2 r = reinterpret_cast<const int2*>(j.R)[i];
    rk[i] = r.x;
    rv[i] = r.y;
    nxt[i] = atomicExch(&head[ej_hash32((uint32_t)r.y) & (nb - 1)], (int)i);
  }
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u;
  for (uint64_t base = (uint64_t)(threadIdx.x >> 5) * 32; base < j.nS; base += PR_THREADS) {
    const uint64_t si = base + lane;
    int2 s = make_int2(0, 0);
    uint32_t c = 0;
    int first = -1;
    if (si < j.nS) {
      s = __ldcs(reinterpret_cast<const int2*>(j.S) + si);
      first = head[ej_hash32((uint32_t)s.y) & (nb - 1)];
      for (int i = first; i >= 0; i = nxt[i]) c += rv[i] == s.y ? 1u : 0u;
    }
    const uint32_t incl = ej_warp_inclusive_sum<uint32_t>(c);
    const uint32_t total = __shfl_sync(EJ_FULL_MASK, incl, 31);
    if (total == 0) continue;
    unsigned long long off = 0;
    if (lane == 0) {
      off = atomicAdd(j.d_count, (unsigned long long)total);
      if (off + total > j.cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
    }
    off = __shfl_sync(EJ_FULL_MASK, off, 0) + (incl - c);
    for (int i = first; c && i >= 0; i = nxt[i]) {
      if (rv[i] != s.y) continue;
      if (off < j.cap) __stcs(reinterpret_cast<int4*>(j.out + off), make_int4(rk[i], s.y, s.x, s.y));
      off++;
    }
  }
}

// The probe of a batch as one launch over a task list, one task per block,
// handed out in list order by the block scheduler: a whole small join (table
// built and probed in shared memory) or one 1024-probe tile of a larger join
// (table from the segmented passes).  The small joins come first, so that no
// large task waits behind them at the end.  (A resident grid pulling tasks
// from an atomic counter measured slower: its loop needs 80 registers a
// thread, three blocks per SM instead of four.)
// (Four blocks per SM: 64 registers a thread; left free it takes 78, three
// blocks, and the 256-instance batch ran 1% slower; at five blocks the
// spills cost 20%.)
__global__ void __launch_bounds__(PR_THREADS, 4)
batch_task_kernel(const BatchJoin* __restrict__ joins, const BatchTask* __restrict__ tasks, ej_dev_status* st) {
  __shared__ int4 smem[PR_WARPS * PW_STAGE_ROWS];  // staging rows, or a small join's table
  static_assert(4 * BX_SMALL_R * sizeof(int32_t) <= sizeof(int4) * PR_WARPS * PW_STAGE_ROWS,
                "a small join's table fits in the staging buffers");
  const BatchTask task = tasks[blockIdx.x];
  const BatchJoin& j = joins[task.join];
  if (task.local == BX_SMALL_TASK)
    batch_small_join(j, smem, st);
  else
    batch_probe_tile(j, task.local, reinterpret_cast<int4(*)[PW_STAGE_ROWS]>(smem), st);
}

}  // namespace

// Plan and launch; counts go to d_counts[i] (device).
static ej_status batch_run(ej_handle* h, const ej_join_desc* jd, uint32_t n, unsigned long long* d_counts) {
  // host-side layout of the batch
  std::vector<BatchJoin> joins(n);
  std::vector<ej_rx_tile> rtiles;
  std::vector<BatchTask> small_tasks, tile_tasks;
  std::vector<unsigned long long> sbase(n);
  uint64_t nr_total = 0, start_total = 0, cells = 0;
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t nR = jd[i].nR, nS = jd[i].nS;
    BatchJoin& b = joins[i];
    b.R = jd[i].R;
    b.S = jd[i].S;
    b.nS = nS;
    b.out = jd[i].out;
    b.cap = jd[i].out_cap;
    b.d_count = d_counts + i;
    b.r_row0 = nr_total;
    b.view.kind = EJ_TABLE_HASH;
    b.view.nR = nR;
    b.view.hb = ej_table_bucket_bits(nR, ej_tuned_bucket_delta(h, nR, BX_BUCKET_DELTA));
    b.nwtiles = (nS + PR_WTILE - 1) / PR_WTILE;
    sbase[i] = start_total;
    if (nR && nR <= BX_SMALL_R) {  // built and probed by one CTA in shared memory
      if (nS) small_tasks.push_back({i, BX_SMALL_TASK});
      continue;
    }
    const uint32_t rt = (uint32_t)((nR + BX_RX_TILE - 1) / BX_RX_TILE);
    for (uint32_t t = 0; t < rt; t++) {
      ej_rx_tile d;
      d.start = nr_total + (uint64_t)t * BX_RX_TILE;
      d.n = (uint32_t)std::min<uint64_t>(BX_RX_TILE, nR - (uint64_t)t * BX_RX_TILE);
      d.cell0 = (uint32_t)(cells + t);
      d.stride = rt;
      d.pad = i;
      d.src = nullptr;
      rtiles.push_back(d);
    }
    cells += (uint64_t)rt * 256;
    start_total += 1ull << b.view.hb;
    const uint32_t nptiles = (uint32_t)((nS + PR_TILE - 1) / PR_TILE);
    for (uint32_t t = 0; t < nptiles; t++) tile_tasks.push_back({i, t});
    nr_total += nR;
  }
  // the task list: small joins first, then every probe tile
  std::vector<BatchTask> tasks(small_tasks);
  tasks.insert(tasks.end(), tile_tasks.begin(), tile_tasks.end());
  if (cells > 0xFFFFFFFFull || nr_total >= 0xFFFFFFFFull)
    return ej_fail(h, EJ_ERR_TOO_LARGE, "batch of %llu R rows is too large", (unsigned long long)nr_total);

  // arena layout
  ej_plan_bytes p;
  const size_t joins_off = p.add(n * sizeof(BatchJoin));
  const size_t rtiles_off = p.add(std::max<size_t>(rtiles.size(), 1) * sizeof(ej_rx_tile));
  const size_t rtiles0_off = p.add(std::max<size_t>(rtiles.size(), 1) * sizeof(ej_rx_tile));
  const size_t tasks_off = p.add(std::max<size_t>(tasks.size(), 1) * sizeof(BatchTask));
  const size_t sbase_off = p.add(n * sizeof(unsigned long long));
  const size_t tmpa_off = p.add(std::max<uint64_t>(nr_total, 1) * sizeof(ej_tuple));
  const size_t tmpb_off = p.add(std::max<uint64_t>(nr_total, 1) * sizeof(ej_tuple));
  const size_t rkey_off = p.add(ej_table_col_bytes(nr_total));
  const size_t rval_off = p.add(ej_table_col_bytes(nr_total));
  const size_t start_off = p.add(start_total * sizeof(uint2));
  ej_radix_plan rp;
  rp.n = nr_total;
  rp.ntiles = (uint32_t)rtiles.size();
  rp.hist_off = p.add(cells * sizeof(uint32_t));
  rp.offs_off = p.add((cells + 1) * sizeof(uint32_t));
  rp.scan_off = p.add(ej_scan_scratch_bytes(cells));
  EJ_TRY(ej_arena_reserve(h, p.bytes));

  char* A = static_cast<char*>(h->arena);
  int32_t* rkey = reinterpret_cast<int32_t*>(A + rkey_off);
  int32_t* rval = reinterpret_cast<int32_t*>(A + rval_off);
  uint2* bucket = reinterpret_cast<uint2*>(A + start_off);
  for (uint32_t i = 0; i < n; i++) {
    BatchJoin& b = joins[i];
    b.view.rkey = rkey + b.r_row0;
    b.view.rval = rval + b.r_row0;
    b.view.voff = (uint32_t)(b.r_row0 & 3u);  // the arena column is 16-byte aligned
    b.view.bucket = bucket + sbase[i];
  }
  // descriptors go up with the batch (stream-ordered copies)
  const size_t jb = n * sizeof(BatchJoin), rb = rtiles.size() * sizeof(ej_rx_tile),
               pb = tasks.size() * sizeof(BatchTask), sb = n * sizeof(unsigned long long);
  EJ_CUDA(h, cudaMemcpyAsync(A + joins_off, joins.data(), jb, cudaMemcpyHostToDevice, h->stream));
  if (rb) EJ_CUDA(h, cudaMemcpyAsync(A + rtiles_off, rtiles.data(), rb, cudaMemcpyHostToDevice, h->stream));
  // the first radix pass reads every join's R where it lies: the same tiles
  // with their source rows
  for (ej_rx_tile& d : rtiles) d.src = joins[d.pad].R + (d.start - joins[d.pad].r_row0);
  if (rb) EJ_CUDA(h, cudaMemcpyAsync(A + rtiles0_off, rtiles.data(), rb, cudaMemcpyHostToDevice, h->stream));
  if (pb) EJ_CUDA(h, cudaMemcpyAsync(A + tasks_off, tasks.data(), pb, cudaMemcpyHostToDevice, h->stream));
  EJ_CUDA(h, cudaMemcpyAsync(A + sbase_off, sbase.data(), sb, cudaMemcpyHostToDevice, h->stream));
  EJ_CUDA(h, cudaMemsetAsync(d_counts, 0, n * sizeof(unsigned long long), h->stream));
  const BatchJoin* djoins = reinterpret_cast<const BatchJoin*>(A + joins_off);
  const ej_rx_tile* drt = reinterpret_cast<const ej_rx_tile*>(A + rtiles_off);
  rp.tiles = drt;

  ej_phase_begin(h);
  if (!rtiles.empty()) {
    ej_tuple* tmp[2] = {reinterpret_cast<ej_tuple*>(A + tmpa_off), reinterpret_cast<ej_tuple*>(A + tmpb_off)};
    ej_radix_plan rp0 = rp;
    rp0.tiles = reinterpret_cast<const ej_rx_tile*>(A + rtiles0_off);
    // pass 0 reads the joins' R arrays in place; its order within a digit is
    // never used (unordered ranking)
    EJ_TRY(ej_partition_pass_src(h, rp0, tmp[0], 0u, 8u));
    EJ_TRY(ej_radix_pass(h, rp, tmp[0], tmp[1], 8u, 8u, EJ_DIGIT_HASH));
    EJ_TRY(ej_radix_pass(h, rp, tmp[1], tmp[0], 16u, 8u, EJ_DIGIT_HASH));
    EJ_TRY(ej_radix_pass_soa(h, rp, tmp[0], rkey, rval, 24u, 8u, EJ_DIGIT_HASH));
  }
  // joins with an empty R keep all-zero bucket starts
  EJ_CUDA(h, cudaMemsetAsync(bucket, 0, start_total * sizeof(uint2), h->stream));
  if (!rtiles.empty()) {
    batch_bucket_start_kernel<<<(unsigned)rtiles.size(), 256, 0, h->stream>>>(
        drt, djoins, bucket, reinterpret_cast<const unsigned long long*>(A + sbase_off));
    EJ_TRY(ej_check_launch(h, "batch_bucket_start_kernel"));
  }
  ej_phase_mark(h, 1);
  ej_phase_mark(h, 2);  // no partition pass: every table of a batch is probed in place
  ej_phase_mark(h, 3);  // one pass: recorded as the write phase
  if (!tasks.empty()) {
    batch_task_kernel<<<(unsigned)tasks.size(), PR_THREADS, 0, h->stream>>>(
        djoins, reinterpret_cast<const BatchTask*>(A + tasks_off), h->d_status);
    EJ_TRY(ej_check_launch(h, "batch_task_kernel"));
  }
  ej_phase_mark(h, 4);
  return EJ_OK;
}

static ej_status batch_check(ej_handle* h, const ej_join_desc* joins, uint32_t n) {
  if (n && !joins) return ej_fail(h, EJ_ERR_INVALID, "joins is NULL");
  for (uint32_t i = 0; i < n; i++) {
    EJ_TRY(ej_check_rel(h, "R", joins[i].R, joins[i].nR));
    EJ_TRY(ej_check_rel(h, "S", joins[i].S, joins[i].nS));
    if (joins[i].out_cap && !joins[i].out) return ej_fail(h, EJ_ERR_INVALID, "join %u: out is NULL", i);
    if (joins[i].out && ((uintptr_t)joins[i].out % 16))
      return ej_fail(h, EJ_ERR_INVALID, "join %u: out must be 16-byte aligned", i);
  }
  return EJ_OK;
}

extern "C" ej_status ej_batch_hash_join_async(ej_handle* h, const ej_join_desc* joins, uint32_t njoins,
                                              uint64_t* d_counts) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(batch_check(h, joins, njoins));
  if (njoins && !d_counts) return ej_fail(h, EJ_ERR_INVALID, "d_counts is NULL");
  if (!njoins) return EJ_OK;
  return batch_run(h, joins, njoins, reinterpret_cast<unsigned long long*>(d_counts));
}

extern "C" ej_status ej_batch_hash_join(ej_handle* h, const ej_join_desc* joins, uint32_t njoins, uint64_t* counts) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(batch_check(h, joins, njoins));
  if (njoins && !counts) return ej_fail(h, EJ_ERR_INVALID, "counts is NULL");
  if (!njoins) return EJ_OK;
  // device counts live in the handle's count area: grow it when needed
  if (njoins > h->batch_counts_cap) {
    EJ_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->d_batch_counts);
    cudaFreeHost(h->h_batch_counts);
    h->d_batch_counts = nullptr;
    h->h_batch_counts = nullptr;
    h->batch_counts_cap = 0;
    EJ_CUDA(h, ej_dev_alloc(&h->d_batch_counts, njoins * sizeof(unsigned long long)));
    EJ_CUDA(h, ej_host_alloc(&h->h_batch_counts, njoins * sizeof(unsigned long long)));
    h->batch_counts_cap = njoins;
  }
  EJ_TRY(batch_run(h, joins, njoins, h->d_batch_counts));
  EJ_CUDA(h, cudaMemcpyAsync(h->h_batch_counts, h->d_batch_counts, njoins * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, h->stream));
  EJ_TRY(ej_finish(h, nullptr));
  bool over = false;
  for (uint32_t i = 0; i < njoins; i++) {
    counts[i] = h->h_batch_counts[i];
    over |= counts[i] > joins[i].out_cap;
  }
  return over ? ej_fail(h, EJ_ERR_CAPACITY, "a join of the batch has more results than its out_cap") : EJ_OK;
}
