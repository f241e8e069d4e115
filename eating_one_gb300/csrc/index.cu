// index.cu - device-resident hash and sort indexes, index joins, the left
// outer join and the 3-way star join.
//
// The reference builds both indexes on the CPU and uploads them (hash index:
// joins/innerJoin_gpu/main_street/inner-idx-bnlj.cc:148-181, `val % 2^24`
// buckets; sort index: joins/innerJoin_gpu/sort_index/main_street/
// inner-idx-bnlj.cc:175-217, recursive quicksort of BUCKET{val,adr}), then
// probes one S tuple per thread (count.cu:16-48 / join_gpu.cu:8-86;
// sort_index join_gpu.cu:10-113).  Here both indexes are built on the device
// with the LSD radix passes of radix.cu: the hash index is the table of
// hash_join.cu (key directory or bucket bounds), the sort index is R sorted by
// val with bucket bounds over value prefixes, (v - vmin) >> vshift, so that a
// probe reads one 8-byte bound pair and the first 8 vals of its bucket
// instead of two binary searches over the table (probe.cuh).
#include <map>
#include <mutex>

#include "ej_device.cuh"
#include "ej_entry.h"
#include "hash_join.cuh"
#include "probe.cuh"
#include "probe_write.cuh"

struct ej_index {
  int kind = EJ_TABLE_HASH;
  int device = 0;
  uint64_t nR = 0;
  int32_t* rkey = nullptr;  // device, owned
  int32_t* rval = nullptr;  // device, owned
  void* aux = nullptr;      // device, owned: key directory, bucket bounds or value buckets
  ej_table_view view;
};

// Index storage comes from a stream-ordered memory pool per device that keeps
// freed memory for the next index (its release threshold is unlimited), so an
// index built after another was freed costs no cudaMalloc (which maps fresh
// pages and synchronises the device: about half of a 2^24-row index build);
// ej_trim returns the pool's unused memory.
static std::mutex g_pool_mu;
static std::map<int, cudaMemPool_t> g_pools;

static cudaError_t index_pool(int device, cudaMemPool_t* pool) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  auto it = g_pools.find(device);
  if (it != g_pools.end()) {
    *pool = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaError_t e = cudaMemPoolCreate(pool, &props);
  if (e != cudaSuccess) return e;
  uint64_t keep = UINT64_MAX;
  e = cudaMemPoolSetAttribute(*pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) {
    cudaMemPoolDestroy(*pool);
    return e;
  }
  g_pools[device] = *pool;
  return cudaSuccess;
}

void ej_index_pool_trim(int device) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  auto it = g_pools.find(device);
  if (it != g_pools.end()) cudaMemPoolTrimTo(it->second, 0);
}

// the index's storage back to the pool, ordered on `stream`
static void index_release(ej_index* ix, cudaStream_t stream) {
  if (ix->rkey) cudaFreeAsync(ix->rkey, stream);
  if (ix->rval) cudaFreeAsync(ix->rval, stream);
  if (ix->aux) cudaFreeAsync(ix->aux, stream);
  delete ix;
}

// ---- index lifecycle ------------------------------------------------------

static ej_status index_build(ej_handle* h, int kind, const ej_tuple* R, uint64_t nR, ej_index** out) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(ej_check_rel(h, "R", R, nR));
  if (!out) return ej_fail(h, EJ_ERR_INVALID, "index out-pointer is NULL");
  *out = nullptr;
  ej_plan_bytes p;
  ej_table_plan_t tp;
  ej_table_plan(p, tp, nR, /*own_storage=*/true, kind, ej_tuned_table_knobs(h, nR));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_index* ix = new ej_index();
  ix->kind = kind;
  ix->device = h->device;
  ix->nR = nR;
  const size_t col = ej_table_col_bytes(nR), aux_bytes = ej_table_aux_bytes(tp);
  cudaMemPool_t pool;
  if (index_pool(h->device, &pool) != cudaSuccess ||
      ej_pool_alloc(reinterpret_cast<void**>(&ix->rkey), col, pool, h->stream) != cudaSuccess ||
      ej_pool_alloc(reinterpret_cast<void**>(&ix->rval), col, pool, h->stream) != cudaSuccess ||
      ej_pool_alloc(&ix->aux, aux_bytes, pool, h->stream) != cudaSuccess) {
    cudaGetLastError();
    index_release(ix, h->stream);
    return ej_fail(h, EJ_ERR_NOMEM, "index storage of %zu bytes could not be allocated", 2 * col + aux_bytes);
  }
  ej_phase_begin(h);
  ej_status st = ej_table_build(h, tp, R, ix->rkey, ix->rval, ix->aux, &ix->view);
  for (int k = 1; k <= EJ_PHASES; k++) ej_phase_mark(h, k);
  uint32_t bits = 1;
  if (st == EJ_OK && ix->view.dir)  // the build's choice: bits = 0 when it took bucket bounds for short runs
    st = cudaMemcpyAsync(&bits, ix->view.dir_bits, sizeof bits, cudaMemcpyDeviceToHost, h->stream) == cudaSuccess
             ? EJ_OK
             : ej_fail(h, EJ_ERR_CUDA, "reading the index header failed");
  if (st == EJ_OK) st = ej_finish(h, nullptr);
  if (st == EJ_OK) ix->view.short_runs = bits == 0 ? 1u : 0u;
  if (st != EJ_OK) {
    cudaStreamSynchronize(h->stream);
    index_release(ix, h->stream);
    return st;
  }
  *out = ix;
  return EJ_OK;
}

extern "C" ej_status ej_hash_index_build(ej_handle* h, const ej_tuple* R, uint64_t nR, ej_index** out) {
  return index_build(h, EJ_TABLE_HASH, R, nR, out);
}

extern "C" ej_status ej_sort_index_build(ej_handle* h, const ej_tuple* R, uint64_t nR, ej_index** out) {
  return index_build(h, EJ_TABLE_SORTED, R, nR, out);
}

extern "C" ej_status ej_index_free(ej_handle* h, ej_index* idx) {
  if (!h || !idx) return EJ_ERR_INVALID;
  EJ_CUDA(h, cudaSetDevice(idx->device));
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));  // no probe of the index is still running on h
  index_release(idx, h->stream);
  return EJ_OK;
}

// ---- index probes ------------------------------------------------------------

static ej_status index_probe(ej_handle* h, const ej_index* ix, const ej_tuple* S, uint64_t nS, bool outer,
                             bool count_only, ej_result* out, uint64_t cap, uint64_t* out_count) {
  EJ_TRY(ej_begin(h));
  if (!ix) return ej_fail(h, EJ_ERR_INVALID, "index is NULL");
  if (ix->device != h->device) return ej_fail(h, EJ_ERR_INVALID, "index lives on another device");
  EJ_TRY(ej_check_rel(h, "S", S, nS));
  if (count_only) {
    if (!out_count) return ej_fail(h, EJ_ERR_INVALID, "out_count is NULL");
  } else {
    EJ_TRY(ej_check_out(h, out, cap, out_count));
  }
  // hash index: partition S by hash when the index outgrows L2; a sorted
  // index is probed in place (S in hash partitions would not follow its order)
  const uint32_t pb = ix->kind == EJ_TABLE_HASH ? ej_probe_partition_bits(h, ix->nR, nS) : 0u;
  ej_plan_bytes p;
  ej_probe_layout L;
  ej_probe_layout_add(p, L, nS, pb, count_only, false, ej_tuned_probe_warps(h, ix->nR));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_phase_mark(h, 1);
  EJ_TRY(ej_probe_exec(h, L, ix->view, S, outer, count_only, out, cap, h->d_words));
  uint64_t count = 0;
  EJ_TRY(ej_finish(h, &count));
  *out_count = count;
  return count_only ? EJ_OK : ej_capacity_result(h, count, cap);
}

extern "C" ej_status ej_index_join(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                                   ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return index_probe(h, idx, S, nS, false, false, out, out_cap, out_count);
}

extern "C" ej_status ej_index_join_count(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                                         uint64_t* out_count) {
  return index_probe(h, idx, S, nS, false, true, nullptr, 0, out_count);
}

extern "C" ej_status ej_index_left_outer_join(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                                              ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return index_probe(h, idx, S, nS, true, false, out, out_cap, out_count);
}

static ej_status build_and_probe(ej_handle* h, int kind, bool outer, const ej_tuple* R, uint64_t nR,
                                 const ej_tuple* S, uint64_t nS, ej_result* out, uint64_t out_cap,
                                 uint64_t* out_count) {
  ej_index* ix = nullptr;
  EJ_TRY(index_build(h, kind, R, nR, &ix));
  const ej_status st = index_probe(h, ix, S, nS, outer, false, out, out_cap, out_count);
  const std::string err = h->last_error;
  ej_index_free(h, ix);
  h->last_error = err;
  return st;
}

extern "C" ej_status ej_hash_index_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                        uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return build_and_probe(h, EJ_TABLE_HASH, false, R, nR, S, nS, out, out_cap, out_count);
}

extern "C" ej_status ej_sort_index_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                        uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return build_and_probe(h, EJ_TABLE_SORTED, false, R, nR, S, nS, out, out_cap, out_count);
}

// Left outer join on a transient hash table held in the arena.
// ---- merge join of a sort index with S in value order ----------------------

namespace {

// Warp tile w: the 128 consecutive rows S[128 w ...] of an S in value order.
// Their matches lie in the index rows between the first row at or above the
// tile's first value and the first row above its last value; lanes 0 and 1
// find those two bounds over the whole index (binary searches), then every
// row's run is searched inside that window only - the merge of the two
// sorted sequences cut into warp-sized pieces along S.  Rows are then written
// as the one-pass probe writes them (one atomic reservation per warp).
__global__ void __launch_bounds__(PR_THREADS)
merge_probe_kernel(const ej_tuple* __restrict__ S, uint64_t nS, ej_table_view t, uint64_t nwtiles,
                   unsigned long long* __restrict__ cursor, ej_result* __restrict__ out, uint64_t cap,
                   ej_dev_status* st) {
  __shared__ int4 stage[PR_WARPS][PW_STAGE_ROWS];
  const unsigned int warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint64_t w = (uint64_t)blockIdx.x * PR_WARPS + warp;
  if (w >= nwtiles) return;
  const uint64_t base = w * PR_WTILE;
  const uint64_t last = min(base + PR_WTILE, nS) - 1;
  const int32_t* rv = t.rval;
  const uint32_t nR = (uint32_t)t.nR;
  // the window [wlo, whi) of the index: lane 0 the lower bound of the first
  // value, lane 1 the upper bound of the last
  uint32_t key1[1] = {0u}, lo1[1] = {0u}, hi1[1] = {nR};
  if (lane < 2) key1[0] = ej_order_key<EJ_TABLE_SORTED>(reinterpret_cast<const int2*>(S)[lane ? last : base].y);
  ej_search_rows<EJ_TABLE_SORTED, 1>(rv, lane < 2 && nR ? 1u : 0u, lane == 1, key1, lo1, hi1);
  const uint32_t wlo = __shfl_sync(EJ_FULL_MASK, lo1[0], 0), whi = __shfl_sync(EJ_FULL_MASK, lo1[0], 1);
  EjProbeWarp pw;
  uint32_t key[PR_ITEMS], lo[PR_ITEMS], hi[PR_ITEMS], active = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * 32 + lane;
    const bool ok = idx < nS;
    pw.s[j] = ok ? __ldcs(reinterpret_cast<const int2*>(S) + idx) : make_int2(0, 0);
    key[j] = ej_order_key<EJ_TABLE_SORTED>(pw.s[j].y);
    lo[j] = wlo;
    hi[j] = whi;
    if (ok && wlo < whi) active |= 1u << j;
  }
  // each run's first row, then (when it holds the value) its end
  ej_search_rows<EJ_TABLE_SORTED, PR_ITEMS>(rv, active, false, key, lo, hi);
  uint32_t found = 0, end[PR_ITEMS], top[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    pw.lo[j] = lo[j];
    pw.cnt[j] = 0;
    end[j] = lo[j] + 1;
    top[j] = whi;
    if ((active >> j & 1u) && lo[j] < whi && __ldg(rv + lo[j]) == pw.s[j].y) {
      pw.cnt[j] = 1;
      if (end[j] < whi) found |= 1u << j;
    }
  }
  ej_search_rows<EJ_TABLE_SORTED, PR_ITEMS>(rv, found, true, key, end, top);
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++)
    if (found >> j & 1u) pw.cnt[j] = end[j] - pw.lo[j];
  unsigned long long mine = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) mine += pw.cnt[j];
  const unsigned long long total = ej_warp_sum<unsigned long long>(mine);
  if (total == 0) return;
  int32_t kk[PR_ITEMS][PW_PREFETCH];
  ej_probe_prefetch<EJ_KEYS_WINDOW>(t, pw, kk);
  unsigned long long off = 0;
  if (lane == 0) {
    off = atomicAdd(cursor, total);
    if (off + total > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
  }
  off = __shfl_sync(EJ_FULL_MASK, off, 0);
  if (off >= cap) return;
  ej_emit_warp(pw, kk, t, off, out, cap, stage[warp]);
}

}  // namespace

extern "C" ej_status ej_index_merge_join(ej_handle* h, const ej_index* ix, const ej_tuple* S, uint64_t nS,
                                         int s_sorted, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  EJ_TRY(ej_begin(h));
  if (!ix) return ej_fail(h, EJ_ERR_INVALID, "index is NULL");
  if (ix->kind != EJ_TABLE_SORTED) return ej_fail(h, EJ_ERR_INVALID, "a merge join needs a sort index");
  if (ix->device != h->device) return ej_fail(h, EJ_ERR_INVALID, "index lives on another device");
  EJ_TRY(ej_check_rel(h, "S", S, nS));
  EJ_TRY(ej_check_out(h, out, out_cap, out_count));
  ej_plan_bytes p;
  ej_radix_plan rp;
  size_t a_off = 0, b_off = 0;
  if (!s_sorted) {  // S in value order: four 8-bit LSD passes into a copy
    a_off = p.add((size_t)(nS ? nS : 1) * sizeof(ej_tuple));
    b_off = p.add((size_t)(nS ? nS : 1) * sizeof(ej_tuple));
    ej_radix_plan_add(p, rp, nS);
  }
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_phase_mark(h, 1);
  const ej_tuple* P = S;
  if (!s_sorted && nS) {
    ej_tuple* a = reinterpret_cast<ej_tuple*>(ej_arena_at(h, a_off));
    ej_tuple* b = reinterpret_cast<ej_tuple*>(ej_arena_at(h, b_off));
    EJ_TRY(ej_partition_pass(h, rp, S, a, 0u, 8u, EJ_DIGIT_VALUE));  // the first pass needs no order
    EJ_TRY(ej_radix_pass(h, rp, a, b, 8u, 8u, EJ_DIGIT_VALUE));
    EJ_TRY(ej_radix_pass(h, rp, b, a, 16u, 8u, EJ_DIGIT_VALUE));
    EJ_TRY(ej_radix_pass(h, rp, a, b, 24u, 8u, EJ_DIGIT_VALUE));
    P = b;
  }
  ej_phase_mark(h, 2);
  ej_phase_mark(h, 3);
  EJ_CUDA(h, cudaMemsetAsync(h->d_words, 0, sizeof(unsigned long long), h->stream));
  const uint64_t nwtiles = (nS + PR_WTILE - 1) / PR_WTILE;
  if (nwtiles) {
    merge_probe_kernel<<<(unsigned)((nwtiles + PR_WARPS - 1) / PR_WARPS), PR_THREADS, 0, h->stream>>>(
        P, nS, ix->view, nwtiles, h->d_words, out, out_cap, h->d_status);
    EJ_TRY(ej_check_launch(h, "merge_probe_kernel"));
  }
  ej_phase_mark(h, 4);
  uint64_t count = 0;
  EJ_TRY(ej_finish(h, &count));
  *out_count = count;
  return ej_capacity_result(h, count, out_cap);
}

extern "C" ej_status ej_left_outer_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                        uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(ej_check_rel(h, "R", R, nR));
  EJ_TRY(ej_check_rel(h, "S", S, nS));
  EJ_TRY(ej_check_out(h, out, out_cap, out_count));
  const uint32_t pb = ej_probe_partition_bits(h, nR, nS);
  ej_plan_bytes p;
  ej_table_plan_t tp;
  ej_table_plan(p, tp, nR, /*own_storage=*/false, EJ_TABLE_HASH, ej_tuned_table_knobs(h, nR), nS);
  ej_probe_layout L;
  ej_probe_layout_add(p, L, nS, pb, /*count_only=*/false, false, ej_tuned_probe_warps(h, nR));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_table_view t;
  EJ_TRY(ej_table_build(h, tp, R, reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rkey_off)),
                        reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rval_off)), ej_arena_at(h, tp.aux_off), &t));
  ej_phase_mark(h, 1);
  EJ_TRY(ej_probe_exec(h, L, t, S, /*outer=*/true, false, out, out_cap, h->d_words));
  uint64_t count = 0;
  EJ_TRY(ej_finish(h, &count));
  *out_count = count;
  return ej_capacity_result(h, count, out_cap);
}

// ---- 3-way star join ------------------------------------------------------------

namespace {

constexpr int ST_THREADS = 256;
constexpr int ST_WARPS = ST_THREADS / 32;
constexpr int ST_ITEMS = 2;  // 40 registers, six blocks per SM (four items: 74, three blocks, 4% slower)
constexpr int ST_WTILE = 32 * ST_ITEMS;  // fact rows per warp

// One pass over the fact rows: lane l of a warp takes rows base + 32j + l
// (j < ST_ITEMS); the runs of all its F1 vals in D1 are found together, then
// those of the F2
// vals of the rows that matched in D2; a row's results are the cross product
// of its two runs.  Each item j gets a warp scan of its result counts, so the
// warp's results are ordered item by item and lanes write consecutive rows
// (one 32-byte row per lane and item when both dimensions have unique keys);
// the warp reserves its rows with one atomic add on the cursor (rows at or
// past cap are dropped, the cursor ends at the exact count).
__global__ void __launch_bounds__(ST_THREADS)
star_fused_kernel(const ej_tuple* __restrict__ F1, const ej_tuple* __restrict__ F2, uint64_t nF, ej_table_view t1,
                  ej_table_view t2, unsigned long long* __restrict__ cursor, ej_star_result* __restrict__ out,
                  uint64_t cap, ej_dev_status* st) {
  const unsigned int lane = threadIdx.x & 31u;
  const uint64_t base = ((uint64_t)blockIdx.x * ST_WARPS + (threadIdx.x >> 5)) * ST_WTILE;
  if (base >= nF) return;
  int2 f1[ST_ITEMS], f2[ST_ITEMS];
  int32_t v1[ST_ITEMS], v2[ST_ITEMS];
  bool ok1[ST_ITEMS], ok2[ST_ITEMS];
#pragma unroll
  for (int j = 0; j < ST_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * 32 + lane;
    ok1[j] = idx < nF;
    f1[j] = ok1[j] ? __ldcs(reinterpret_cast<const int2*>(F1) + idx) : make_int2(0, 0);
    f2[j] = ok1[j] ? __ldcs(reinterpret_cast<const int2*>(F2) + idx) : make_int2(0, 0);
    v1[j] = f1[j].y;
    v2[j] = f2[j].y;
  }
  uint32_t lo1[ST_ITEMS], c1[ST_ITEMS], lo2[ST_ITEMS], c2[ST_ITEMS];
  ej_find_runs<EJ_TABLE_HASH, ST_ITEMS>(t1, v1, ok1, lo1, c1);
#pragma unroll
  for (int j = 0; j < ST_ITEMS; j++) ok2[j] = c1[j] != 0;
  ej_find_runs<EJ_TABLE_HASH, ST_ITEMS>(t2, v2, ok2, lo2, c2);
  unsigned long long excl[ST_ITEMS], all = 0;
#pragma unroll
  for (int j = 0; j < ST_ITEMS; j++) {
    const unsigned long long n = (unsigned long long)c1[j] * c2[j];
    const unsigned long long incl = ej_warp_inclusive_sum<unsigned long long>(n);
    excl[j] = all + incl - n;
    all += __shfl_sync(EJ_FULL_MASK, incl, 31);
  }
  if (all == 0) return;
  unsigned long long off = 0;
  if (lane == 0) {
    off = atomicAdd(cursor, all);
    if (off + all > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
  }
  off = __shfl_sync(EJ_FULL_MASK, off, 0);
  if (off >= cap) return;
#pragma unroll
  for (int j = 0; j < ST_ITEMS; j++) {
    if (!c2[j]) continue;
    unsigned long long pos = off + excl[j];
    for (uint32_t a = 0; a < c1[j]; a++) {
      const int32_t k1 = __ldg(t1.rkey + lo1[j] + a);
      for (uint32_t b = 0; b < c2[j]; b++) {
        if (pos < cap) {
          int4* o = reinterpret_cast<int4*>(out + pos);
          __stcs(o, make_int4(k1, f1[j].y, f1[j].x, f1[j].y));
          __stcs(o + 1, make_int4(__ldg(t2.rkey + lo2[j] + b), f2[j].y, f2[j].x, f2[j].y));
        }
        pos++;
      }
    }
  }
}

}  // namespace

extern "C" ej_status ej_star_join3(ej_handle* h, const ej_tuple* F1, const ej_tuple* F2, uint64_t nF,
                                   const ej_tuple* D1, uint64_t nD1, const ej_tuple* D2, uint64_t nD2,
                                   ej_star_result* out, uint64_t out_cap, uint64_t* out_count) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(ej_check_rel(h, "F1", F1, nF));
  EJ_TRY(ej_check_rel(h, "F2", F2, nF));
  EJ_TRY(ej_check_rel(h, "D1", D1, nD1));
  EJ_TRY(ej_check_rel(h, "D2", D2, nD2));
  EJ_TRY(ej_check_out(h, out, out_cap, out_count));
  ej_plan_bytes p;
  ej_table_plan_t tp1, tp2;
  ej_table_knobs k1 = ej_tuned_table_knobs(h, nD1), k2 = ej_tuned_table_knobs(h, nD2);
  k1.delta = k2.delta = 0;  // the star join's dimension tables keep the default load factor
  ej_table_plan(p, tp1, nD1, false, EJ_TABLE_HASH, k1, nF);
  ej_table_plan(p, tp2, nD2, false, EJ_TABLE_HASH, k2, nF);
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_table_view t1, t2;
  EJ_TRY(ej_table_build(h, tp1, D1, reinterpret_cast<int32_t*>(ej_arena_at(h, tp1.rkey_off)),
                        reinterpret_cast<int32_t*>(ej_arena_at(h, tp1.rval_off)), ej_arena_at(h, tp1.aux_off), &t1));
  EJ_TRY(ej_table_build(h, tp2, D2, reinterpret_cast<int32_t*>(ej_arena_at(h, tp2.rkey_off)),
                        reinterpret_cast<int32_t*>(ej_arena_at(h, tp2.rval_off)), ej_arena_at(h, tp2.aux_off), &t2));
  ej_phase_mark(h, 1);
  ej_phase_mark(h, 2);
  ej_phase_mark(h, 3);  // one pass: recorded as the write phase
  EJ_CUDA(h, cudaMemsetAsync(h->d_words, 0, sizeof(unsigned long long), h->stream));  // the row cursor
  const uint64_t blocks = (nF + (uint64_t)ST_WARPS * ST_WTILE - 1) / ((uint64_t)ST_WARPS * ST_WTILE);
  if (blocks > 0x7FFFFFFFull) return ej_fail(h, EJ_ERR_INVALID, "star join: %llu fact rows is too many",
                                             (unsigned long long)nF);
  if (blocks) {
    star_fused_kernel<<<(unsigned)blocks, ST_THREADS, 0, h->stream>>>(F1, F2, nF, t1, t2, h->d_words, out, out_cap,
                                                                     h->d_status);
    EJ_TRY(ej_check_launch(h, "star_fused_kernel"));
  }
  ej_phase_mark(h, 4);
  uint64_t count = 0;
  EJ_TRY(ej_finish(h, &count));
  *out_count = count;
  return ej_capacity_result(h, count, out_cap);
}
