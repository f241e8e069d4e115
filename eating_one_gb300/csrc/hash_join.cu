// hash_join.cu - bucketised hash table on R and the count -> scan -> write probe.
//
// Reference path replaced (joins/hashJoin_gpu/main_street): radix-partition
// both relations into ~|R|/64 partitions, split left partitions into 256-tuple
// chunks on the host, then `count` and `join` compare every chunk tuple with
// every tuple of the matching right partition (join_gpu.cu:9-113) - O(256*|Rp|)
// compares per block, and the write pass repeats all of them.
//
// Here:
//   build  R is sorted stably by bucket id = top `hb` bits of hash32(val)
//          (LSD radix passes, radix.cu), and start[b] marks where bucket b
//          begins - the layout of the reference's hash index (Bucket grouped by
//          bucket + Buck_array offsets, joins/CPU_JOIN/inner_cpu/
//          inner-idx-bnlj.cc:142-166), built on the device.
//   S      when the table does not fit in L2, S is radix-partitioned once by
//          the top `pb` hash bits, so probes of consecutive tiles touch one
//          table region at a time and hit L2; otherwise S is probed in place.
//   probe  count kernel (matches per 2048-tuple tile) -> look-back scan of the
//          tile counts (64-bit) -> write kernel (block scan of per-thread
//          counts, rows written at tile offset + thread prefix).  Output order
//          is deterministic: tile, thread, item, then R order.
// The same probe kernels serve the sort index (ej_table_view kind
// EJ_TABLE_SORTED: the matching run is found by binary search) and the left
// outer join (OUTER: an unmatched probe row yields one NULL-extended row).
#include "ej_device.cuh"
#include "hash_join.cuh"

namespace {

constexpr int PR_THREADS = 256;
constexpr int PR_ITEMS = 8;
constexpr int PR_TILE = PR_THREADS * PR_ITEMS;

__device__ __forceinline__ uint32_t bucket_of(int32_t val, uint32_t bshift) {
  return ej_hash32((uint32_t)val) >> bshift;
}

// start[b] = first position of bucket b in the bucket-sorted relation, b in [0, 2^hb].
__global__ void bucket_start_kernel(const ej_tuple* __restrict__ rs, uint64_t nR, uint32_t* __restrict__ start,
                                    uint32_t hb) {
  const uint32_t bshift = 32u - hb;
  const int64_t nbuckets = (int64_t)1 << hb;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nR;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t cur = i < nR ? (int64_t)bucket_of(rs[i].val, bshift) : nbuckets;
    const int64_t prev = i > 0 ? (int64_t)bucket_of(rs[i - 1].val, bshift) : -1;
    for (int64_t b = prev + 1; b <= cur; b++) start[b] = (uint32_t)i;
  }
}

// fence[i] = rs[i * EJ_FENCE_STRIDE].val of a val-sorted relation
__global__ void fence_kernel(const ej_tuple* __restrict__ rs, uint64_t nR, int32_t* __restrict__ fence,
                             uint32_t nfence) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfence; i += gridDim.x * blockDim.x)
    fence[i] = rs[(uint64_t)i * EJ_FENCE_STRIDE].val;
}

// ---- where a probe value's candidates lie ------------------------------------

template <int KIND>
struct Range;

template <>
struct Range<EJ_TABLE_HASH> {
  // candidates: the whole bucket; callers compare val
  static __device__ __forceinline__ void find(const ej_table_view& t, int32_t v, uint32_t& lo, uint32_t& hi) {
    const uint32_t b = bucket_of(v, 32u - t.hb);
    lo = __ldg(t.start + b);
    hi = __ldg(t.start + b + 1);
  }
};

// first index in [lo, hi) of the val-sorted relation whose val is >= v
// (STRICT: > v), hi when there is none
template <bool STRICT>
__device__ __forceinline__ uint32_t sorted_bound(const int* vals2, uint32_t lo, uint32_t hi, int32_t v) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    const int32_t x = __ldg(vals2 + 2 * (uint64_t)mid);
    if (STRICT ? (x <= v) : (x < v)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <bool STRICT>
__device__ __forceinline__ uint32_t fenced_bound(const ej_table_view& t, int32_t v) {
  // fence search: first fence entry f with fence[f] >= v (STRICT: > v)
  uint32_t flo = 0, fhi = t.nfence;
  while (flo < fhi) {
    const uint32_t mid = (flo + fhi) >> 1;
    const int32_t x = __ldg(t.fence + mid);
    if (STRICT ? (x <= v) : (x < v)) flo = mid + 1; else fhi = mid;
  }
  if (flo == 0) return 0;
  const uint64_t seg_lo = (uint64_t)(flo - 1) * EJ_FENCE_STRIDE;
  const uint64_t seg_hi = min((uint64_t)flo * EJ_FENCE_STRIDE, t.nR);
  return sorted_bound<STRICT>(reinterpret_cast<const int*>(t.rs) + 1, (uint32_t)seg_lo, (uint32_t)seg_hi, v);
}

template <>
struct Range<EJ_TABLE_SORTED> {
  // candidates: exactly the run of equal vals
  static __device__ __forceinline__ void find(const ej_table_view& t, int32_t v, uint32_t& lo, uint32_t& hi) {
    lo = fenced_bound<false>(t, v);
    hi = fenced_bound<true>(t, v);
  }
};

// ---- count and write kernels ------------------------------------------------------

template <int KIND, bool OUTER>
__global__ void __launch_bounds__(PR_THREADS)
probe_count_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t,
                   unsigned long long* __restrict__ tile_count) {
  __shared__ unsigned long long warp_tmp[PR_THREADS / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * PR_TILE;
  const int* pv = reinterpret_cast<const int*>(P) + 1;
  const int* rv = reinterpret_cast<const int*>(t.rs) + 1;
  int v[PR_ITEMS];
  uint32_t lo[PR_ITEMS], hi[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    v[j] = idx < nP ? __ldcs(pv + 2 * idx) : 0;
  }
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    lo[j] = hi[j] = 0;
    if (idx < nP) Range<KIND>::find(t, v[j], lo[j], hi[j]);
  }
  unsigned long long c = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    uint32_t m;
    if (KIND == EJ_TABLE_SORTED) {
      m = hi[j] - lo[j];
    } else {
      m = 0;
      for (uint32_t i = lo[j]; i < hi[j]; i++) m += (__ldg(rv + 2 * (uint64_t)i) == v[j]);
    }
    if (OUTER && idx < nP && m == 0) m = 1;
    c += m;
  }
  unsigned long long total;
  ej_block_exclusive_sum<PR_THREADS, unsigned long long>(c, warp_tmp, &total);
  if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

__device__ __forceinline__ void store_row(ej_result* out, uint64_t pos, int32_t rk, int32_t rv, int32_t lk,
                                          int32_t lv) {
  __stcs(reinterpret_cast<int4*>(out + pos), make_int4(rk, rv, lk, lv));
}

template <int KIND, bool OUTER>
__global__ void __launch_bounds__(PR_THREADS)
probe_write_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t,
                   const unsigned long long* __restrict__ tile_off, uint64_t ntiles, ej_result* __restrict__ out,
                   uint64_t cap, ej_dev_status* st) {
  __shared__ unsigned long long warp_tmp[PR_THREADS / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * PR_TILE;
  const int* rv = reinterpret_cast<const int*>(t.rs) + 1;
  int2 s[PR_ITEMS];
  uint32_t lo[PR_ITEMS], hi[PR_ITEMS], m[PR_ITEMS];
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    s[j] = idx < nP ? __ldcs(reinterpret_cast<const int2*>(P) + idx) : make_int2(0, 0);
  }
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    lo[j] = hi[j] = 0;
    if (idx < nP) Range<KIND>::find(t, s[j].y, lo[j], hi[j]);
  }
  unsigned long long c = 0;
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    uint32_t k;
    if (KIND == EJ_TABLE_SORTED) {
      k = hi[j] - lo[j];
    } else {
      k = 0;
      for (uint32_t i = lo[j]; i < hi[j]; i++) k += (__ldg(rv + 2 * (uint64_t)i) == s[j].y);
    }
    m[j] = k;
    c += (OUTER && idx < nP && k == 0) ? 1u : k;
  }
  unsigned long long total;
  unsigned long long pos = ej_block_exclusive_sum<PR_THREADS, unsigned long long>(c, warp_tmp, &total);
  pos += tile_off[blockIdx.x];
  if (blockIdx.x == 0 && threadIdx.x == 0 && tile_off[ntiles] > cap) ej_set_status(st, EJ_ERR_CAPACITY, 0u);
#pragma unroll
  for (int j = 0; j < PR_ITEMS; j++) {
    const uint64_t idx = base + (uint64_t)j * PR_THREADS + threadIdx.x;
    if (idx >= nP) continue;
    if (OUTER && m[j] == 0) {
      if (pos < cap) store_row(out, pos, EJ_NULL_KEY, EJ_NULL_KEY, s[j].x, s[j].y);
      pos++;
      continue;
    }
    if (m[j] == 0) continue;
    for (uint32_t i = lo[j]; i < hi[j]; i++) {
      const int2 r = __ldg(reinterpret_cast<const int2*>(t.rs) + i);
      if (KIND == EJ_TABLE_SORTED || r.y == s[j].y) {
        if (pos < cap) store_row(out, pos, r.x, r.y, s[j].x, s[j].y);
        pos++;
      }
    }
  }
}

template <int KIND, bool OUTER>
ej_status launch_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       unsigned long long* tcount) {
  probe_count_kernel<KIND, OUTER><<<(unsigned)pp.ntiles, PR_THREADS, 0, h->stream>>>(P, pp.nP, t, tcount);
  return ej_check_launch(h, "probe_count_kernel");
}

template <int KIND, bool OUTER>
ej_status launch_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       const unsigned long long* toff, ej_result* out, uint64_t cap) {
  probe_write_kernel<KIND, OUTER><<<(unsigned)pp.ntiles, PR_THREADS, 0, h->stream>>>(P, pp.nP, t, toff, pp.ntiles,
                                                                                    out, cap, h->d_status);
  return ej_check_launch(h, "probe_write_kernel");
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

void ej_table_plan(ej_plan_bytes& p, ej_table_plan_t& tp, uint64_t nR, bool own_storage, int kind, int delta) {
  tp.kind = kind;
  tp.nR = nR;
  tp.hb = kind == EJ_TABLE_HASH ? ej_table_bucket_bits(nR, delta) : 32u;
  tp.passes = (tp.hb + 7) / 8;
  tp.nfence = (uint32_t)((nR + EJ_FENCE_STRIDE - 1) / EJ_FENCE_STRIDE);
  const size_t tuples = (size_t)(nR ? nR : 1) * sizeof(ej_tuple);
  if (!own_storage) {
    tp.rs_off = p.add(tuples);
    if (kind == EJ_TABLE_HASH) tp.start_off = p.add(((size_t(1) << tp.hb) + 1) * sizeof(uint32_t));
    else tp.start_off = p.add((size_t)(tp.nfence ? tp.nfence : 1) * sizeof(int32_t));
  }
  tp.tmp_off = p.add(tuples);
  ej_radix_plan_add(p, tp.rplan, nR);
}

size_t ej_table_bytes(uint64_t nR, int delta) {
  const uint32_t hb = ej_table_bucket_bits(nR, delta);
  return (size_t)nR * sizeof(ej_tuple) + ((size_t(1) << hb) + 1) * sizeof(uint32_t);
}

ej_status ej_table_build(ej_handle* h, const ej_table_plan_t& tp, const ej_tuple* R, ej_tuple* rs, void* aux,
                         ej_table_view* view) {
  ej_tuple* tmp = reinterpret_cast<ej_tuple*>(ej_arena_at(h, tp.tmp_off));
  // LSD passes over the key, least significant digit first; the last pass
  // writes rs.  Hash tables sort by the hb-bit bucket id (bits [32-hb, 32) of
  // the hash); sorted indexes by all 32 bits of the order-preserving value.
  const uint32_t lo_bit = 32u - tp.hb;
  const int digit_kind = tp.kind == EJ_TABLE_HASH ? EJ_DIGIT_HASH : EJ_DIGIT_VALUE;
  const ej_tuple* src = R;
  uint32_t done = 0;
  for (uint32_t p = 0; p < tp.passes; p++) {
    const uint32_t remaining = tp.hb - done;
    const uint32_t bits = (remaining + (tp.passes - p) - 1) / (tp.passes - p);
    ej_tuple* dst = ((tp.passes - 1 - p) % 2 == 0) ? rs : tmp;
    if (tp.nR) EJ_TRY(ej_radix_pass(h, tp.rplan, src, dst, lo_bit + done, bits, digit_kind));
    src = dst;
    done += bits;
  }
  view->kind = tp.kind;
  view->rs = rs;
  view->nR = tp.nR;
  view->hb = tp.hb;
  if (tp.kind == EJ_TABLE_HASH) {
    uint32_t* start = static_cast<uint32_t*>(aux);
    const uint64_t work = tp.nR + 1;
    const unsigned blocks = (unsigned)std::min<uint64_t>((work + 255) / 256, (uint64_t)h->num_sms * 16);
    bucket_start_kernel<<<blocks, 256, 0, h->stream>>>(rs, tp.nR, start, tp.hb);
    EJ_TRY(ej_check_launch(h, "bucket_start_kernel"));
    view->start = start;
  } else {
    int32_t* fence = static_cast<int32_t*>(aux);
    if (tp.nfence) {
      const unsigned blocks = (unsigned)std::min<uint64_t>((tp.nfence + 255) / 256, (uint64_t)h->num_sms * 16);
      fence_kernel<<<blocks, 256, 0, h->stream>>>(rs, tp.nR, fence, tp.nfence);
      EJ_TRY(ej_check_launch(h, "fence_kernel"));
    }
    view->fence = fence;
    view->nfence = tp.nfence;
  }
  return EJ_OK;
}

// ---- probe --------------------------------------------------------------

uint64_t ej_probe_tiles(uint64_t nP) { return (nP + PR_TILE - 1) / PR_TILE; }

void ej_probe_plan(ej_plan_bytes& p, ej_probe_plan_t& pp, uint64_t nP) {
  pp.nP = nP;
  pp.ntiles = ej_probe_tiles(nP);
  pp.count_off = p.add((pp.ntiles + 1) * sizeof(unsigned long long));
  pp.off_off = p.add((pp.ntiles + 1) * sizeof(unsigned long long));
  pp.scan_off = p.add(ej_scan_scratch_bytes(pp.ntiles));
}

ej_status ej_probe_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, unsigned long long* d_count) {
  unsigned long long* tcount = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.count_off));
  unsigned long long* toff = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.off_off));
  if (pp.ntiles) {
    if (t.kind == EJ_TABLE_HASH)
      EJ_TRY(outer ? launch_count<EJ_TABLE_HASH, true>(h, pp, P, t, tcount)
                   : launch_count<EJ_TABLE_HASH, false>(h, pp, P, t, tcount));
    else
      EJ_TRY(outer ? launch_count<EJ_TABLE_SORTED, true>(h, pp, P, t, tcount)
                   : launch_count<EJ_TABLE_SORTED, false>(h, pp, P, t, tcount));
  }
  EJ_TRY(ej_scan_u64_u64(h, tcount, pp.ntiles, toff, ej_arena_at(h, pp.scan_off)));
  if (d_count)
    EJ_CUDA(h, cudaMemcpyAsync(d_count, toff + pp.ntiles, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                               h->stream));
  return EJ_OK;
}

ej_status ej_probe_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, ej_result* out, uint64_t cap) {
  if (!pp.ntiles) return EJ_OK;
  const unsigned long long* toff = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.off_off));
  if (t.kind == EJ_TABLE_HASH)
    return outer ? launch_write<EJ_TABLE_HASH, true>(h, pp, P, t, toff, out, cap)
                 : launch_write<EJ_TABLE_HASH, false>(h, pp, P, t, toff, out, cap);
  return outer ? launch_write<EJ_TABLE_SORTED, true>(h, pp, P, t, toff, out, cap)
               : launch_write<EJ_TABLE_SORTED, false>(h, pp, P, t, toff, out, cap);
}

// ---- partition bits for the probe side ------------------------------------

uint32_t ej_probe_partition_bits(const ej_handle* h, uint64_t nR, uint64_t nS) {
  (void)nS;
  const uint32_t hb = ej_table_bucket_bits(nR, h->opt_bucket_delta);
  if (h->opt_partition_bits >= 0) return std::min<uint32_t>((uint32_t)h->opt_partition_bits, std::min(hb, 8u));
  const double table = (double)ej_table_bytes(nR, h->opt_bucket_delta);
  const double l2 = (double)(h->l2_bytes ? h->l2_bytes : (size_t)126 << 20);
  if (table <= l2 / 4.0) return 0;  // the whole table stays L2-resident
  // one partition's table region should be a few MB so that the partitions in
  // flight (about two) share L2 with the streaming probe and output traffic
  uint32_t pb = ej_ceil_log2((uint64_t)(table / (l2 / 32.0)) + 1);
  if (pb > 8) pb = 8;
  if (pb > hb) pb = hb;
  return pb;
}

// ---- probe drivers -------------------------------------------------------

void ej_probe_layout_add(ej_plan_bytes& p, ej_probe_layout& L, uint64_t nS, uint32_t pb) {
  L.pb = pb;
  if (pb) {
    L.spart_off = p.add((size_t)nS * sizeof(ej_tuple));
    ej_radix_plan_add(p, L.splan, nS);
  }
  ej_probe_plan(p, L.pp, nS);
}

// Partition S (when the layout says so), count, scan and write; records
// phase marks 2..4 (the caller has begun the set and marked the build).  The arena
// must already hold the layout (reserved together with anything the table
// placed there, so that no reservation moves a built table).
ej_status ej_probe_exec(ej_handle* h, const ej_probe_layout& L, const ej_table_view& t, const ej_tuple* S,
                        bool outer, bool count_only, ej_result* out, uint64_t out_cap,
                        unsigned long long* d_count) {
  const ej_tuple* P = S;
  if (L.pb) {
    ej_tuple* spart = reinterpret_cast<ej_tuple*>(ej_arena_at(h, L.spart_off));
    EJ_TRY(ej_radix_pass(h, L.splan, S, spart, 32u - L.pb, L.pb));
    P = spart;
  }
  ej_phase_mark(h, 2);
  EJ_TRY(ej_probe_count(h, L.pp, P, t, outer, d_count));
  ej_phase_mark(h, 3);
  if (!count_only) EJ_TRY(ej_probe_write(h, L.pp, P, t, outer, out, out_cap));
  ej_phase_mark(h, 4);
  return EJ_OK;
}

ej_status ej_hash_join_run(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                           ej_result* out, uint64_t out_cap, unsigned long long* d_count, int mode) {
  // mode: 0 = partition S when the planner says so, 1 = never partition S, 2 = count only
  const uint32_t pb = (mode == 1) ? 0u : ej_probe_partition_bits(h, nR, nS);
  ej_plan_bytes p;
  ej_table_plan_t tp;
  ej_table_plan(p, tp, nR, /*own_storage=*/false, EJ_TABLE_HASH, h->opt_bucket_delta);
  ej_probe_layout L;
  ej_probe_layout_add(p, L, nS, pb);
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_tuple* rs = reinterpret_cast<ej_tuple*>(ej_arena_at(h, tp.rs_off));
  ej_table_view t;
  EJ_TRY(ej_table_build(h, tp, R, rs, ej_arena_at(h, tp.start_off), &t));
  ej_phase_mark(h, 1);
  return ej_probe_exec(h, L, t, S, /*outer=*/false, mode == 2, out, out_cap, d_count);
}
