// hash_join.cu - the table build and the probe (count, and write with
// decoupled look-back) shared by every join that probes R.
//
// Reference path replaced (joins/hashJoin_gpu/main_street): radix-partition
// both relations into ~|R|/64 partitions, split left partitions into 256-tuple
// chunks on the host, then `count` and `join` compare every chunk tuple with
// every tuple of the matching right partition (join_gpu.cu:9-113) - O(256*|Rp|)
// compares per block, and the write pass repeats all of them.
//
// Here:
//   build  R is sorted by hash32(val) with four 8-bit LSD radix passes
//          (radix.cu); the last pass writes it as two arrays rkey[]/rval[],
//          and start[b] marks where bucket b (top hb hash bits) begins - the
//          grouped layout of the reference's hash index (Bucket + Buck_array,
//          joins/CPU_JOIN/inner_cpu/inner-idx-bnlj.cc:142-166), built on the
//          device.  The hash is a bijection, so equal keys are one contiguous
//          run and a probe yields (run start, run length).
//   S      when the table does not fit in L2, S is radix-partitioned once by
//          the top pb hash bits, so consecutive probe tiles touch one table
//          region at a time and hit L2; otherwise S is probed in place.
//   write  one kernel per join: each 1024-probe tile finds its runs, scans
//          its counts, takes its output offset from the preceding tiles by
//          decoupled look-back (tiles claim ids in order), then expands the
//          runs into rows staged in shared memory and written out as
//          coalesced 16-byte streaming stores (probe_write.cuh).  The
//          separate count kernel + scan serve the *_count entry points.  Output order is deterministic:
//          tile, probe, then R run order.
// The same kernels serve the sort index (runs by binary search) and the left
// outer join (OUTER: a probe without matches yields one NULL-extended row).
#include "ej_device.cuh"
#include "hash_join.cuh"
#include "probe.cuh"
#include "probe_write.cuh"

namespace {


// start[b] = first position of bucket b in the hash-sorted table, b in [0, 2^hb].
__global__ void bucket_start_kernel(const int32_t* __restrict__ rval, uint64_t nR, uint32_t* __restrict__ start,
                                    uint32_t hb) {
  const int64_t nbuckets = (int64_t)1 << hb;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nR;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t cur = i < nR ? (int64_t)ej_bucket_of(rval[i], hb) : nbuckets;
    const int64_t prev = i > 0 ? (int64_t)ej_bucket_of(rval[i - 1], hb) : -1;
    for (int64_t b = prev + 1; b <= cur; b++) start[b] = (uint32_t)i;
  }
}

// fence[i] = rval[i * EJ_FENCE_STRIDE] of a val-sorted table
__global__ void fence_kernel(const int32_t* __restrict__ rval, int32_t* __restrict__ fence, uint32_t nfence) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfence; i += gridDim.x * blockDim.x)
    fence[i] = rval[(uint64_t)i * EJ_FENCE_STRIDE];
}

// ---- count (for the *_count entry points) ---------------------------------------
// Each warp tile's row total; a scan of the totals gives the join's size.

template <int KIND, bool OUTER>
__global__ void __launch_bounds__(PR_THREADS)
probe_count_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t, unsigned long long* __restrict__ wcount,
                   uint64_t nwtiles) {
  const uint64_t w = (uint64_t)blockIdx.x * PR_WARPS + (threadIdx.x >> 5);
  if (w >= nwtiles) return;
  const unsigned long long total = ej_probe_count_warp<KIND, OUTER>(P, w * PR_WTILE, nP, t);
  if ((threadIdx.x & 31u) == 0) wcount[w] = total;
}

// ---- write with decoupled look-back ---------------------------------------------

template <int KIND, bool OUTER>
__global__ void __launch_bounds__(PR_THREADS, 3)
probe_write_kernel(const ej_tuple* __restrict__ P, uint64_t nP, ej_table_view t, unsigned long long* lb_status,
                   unsigned int* tile_ctr, uint64_t ntiles, ej_result* __restrict__ out, uint64_t cap,
                   unsigned long long* d_total, ej_dev_status* st) {
  extern __shared__ __align__(16) unsigned char pw_smem_raw[];
  PwSmem& sm = *reinterpret_cast<PwSmem*>(pw_smem_raw);
  if (threadIdx.x == 0) sm.tile = atomicAdd(tile_ctr, 1u);  // tiles claim ids in launch order (look-back progress)
  __syncthreads();
  const uint64_t tile = sm.tile;
  ej_probe_write_tile<KIND, OUTER>(sm, P, tile * PR_TILE, nP, t, lb_status, tile, tile == ntiles - 1, out, cap,
                                   d_total, st);
}

template <int KIND, bool OUTER>
ej_status launch_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       unsigned long long* wcount) {
  probe_count_kernel<KIND, OUTER><<<(unsigned)pp.ntiles, PR_THREADS, 0, h->stream>>>(P, pp.nP, t, wcount, pp.nwtiles);
  return ej_check_launch(h, "probe_count_kernel");
}

template <int KIND, bool OUTER>
ej_status launch_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                       ej_result* out, uint64_t cap, unsigned long long* d_total) {
  unsigned long long* lb = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.lb_off));
  unsigned int* ctr = reinterpret_cast<unsigned int*>(lb + pp.ntiles);
  EJ_CUDA(h, cudaMemsetAsync(lb, 0, pp.ntiles * sizeof(unsigned long long) + 16, h->stream));
  auto k = probe_write_kernel<KIND, OUTER>;
  EJ_CUDA(h, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PwSmem)));
  k<<<(unsigned)pp.ntiles, PR_THREADS, sizeof(PwSmem), h->stream>>>(P, pp.nP, t, lb, ctr, pp.ntiles, out, cap,
                                                                     d_total, h->d_status);
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

size_t ej_table_aux_bytes(const ej_table_plan_t& tp) {
  return tp.kind == EJ_TABLE_HASH ? ((size_t(1) << tp.hb) + 1) * sizeof(uint32_t)
                                  : (size_t)(tp.nfence ? tp.nfence : 1) * sizeof(int32_t);
}

size_t ej_table_col_bytes(uint64_t nR) { return (size_t)(nR + EJ_TABLE_PAD) * sizeof(int32_t); }

void ej_table_plan(ej_plan_bytes& p, ej_table_plan_t& tp, uint64_t nR, bool own_storage, int kind, int delta) {
  tp.kind = kind;
  tp.nR = nR;
  tp.hb = kind == EJ_TABLE_HASH ? ej_table_bucket_bits(nR, delta) : 32u;
  tp.passes = 4;  // all 32 key bits: equal keys end up adjacent
  tp.nfence = (uint32_t)((nR + EJ_FENCE_STRIDE - 1) / EJ_FENCE_STRIDE);
  if (!own_storage) {
    tp.rkey_off = p.add(ej_table_col_bytes(nR));
    tp.rval_off = p.add(ej_table_col_bytes(nR));
    tp.aux_off = p.add(ej_table_aux_bytes(tp));
  }
  const size_t tuples = (size_t)(nR ? nR : 1) * sizeof(ej_tuple);
  tp.tmp_a_off = p.add(tuples);
  tp.tmp_b_off = p.add(tuples);
  ej_radix_plan_add(p, tp.rplan, nR);
}

size_t ej_table_bytes(uint64_t nR, int delta) {
  const uint32_t hb = ej_table_bucket_bits(nR, delta);
  return (size_t)nR * sizeof(ej_tuple) + ((size_t(1) << hb) + 1) * sizeof(uint32_t);
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
  for (uint32_t p = 0; p < tp.passes && tp.nR; p++) {
    const uint32_t shift = 8u * p;
    if (p + 1 == tp.passes) {
      EJ_TRY(ej_radix_pass_soa(h, tp.rplan, src, rkey, rval, shift, 8u, digit_kind));
    } else {
      EJ_TRY(ej_radix_pass(h, tp.rplan, src, tmp[p & 1], shift, 8u, digit_kind));
      src = tmp[p & 1];
    }
  }
  view->kind = tp.kind;
  view->rkey = rkey;
  view->rval = rval;
  view->nR = tp.nR;
  view->hb = tp.hb;
  if (tp.kind == EJ_TABLE_HASH) {
    uint32_t* start = static_cast<uint32_t*>(aux);
    const uint64_t work = tp.nR + 1;
    const unsigned blocks = (unsigned)std::min<uint64_t>((work + 255) / 256, (uint64_t)h->num_sms * 16);
    bucket_start_kernel<<<blocks, 256, 0, h->stream>>>(rval, tp.nR, start, tp.hb);
    EJ_TRY(ej_check_launch(h, "bucket_start_kernel"));
    view->start = start;
  } else {
    int32_t* fence = static_cast<int32_t*>(aux);
    if (tp.nfence) {
      const unsigned blocks = (unsigned)std::min<uint64_t>((tp.nfence + 255) / 256, (uint64_t)h->num_sms * 16);
      fence_kernel<<<blocks, 256, 0, h->stream>>>(rval, fence, tp.nfence);
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
  pp.nwtiles = (nP + PR_WTILE - 1) / PR_WTILE;
  pp.count_off = p.add((pp.nwtiles + 1) * sizeof(unsigned long long));
  pp.off_off = p.add((pp.nwtiles + 1) * sizeof(unsigned long long));
  pp.scan_off = p.add(ej_scan_scratch_bytes(pp.nwtiles));
  pp.lb_off = p.add(pp.ntiles * sizeof(unsigned long long) + 16);
}

ej_status ej_probe_count(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, unsigned long long* d_count) {
  unsigned long long* wcount = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.count_off));
  unsigned long long* woff = reinterpret_cast<unsigned long long*>(ej_arena_at(h, pp.off_off));
  if (pp.ntiles) {
    if (t.kind == EJ_TABLE_HASH)
      EJ_TRY(outer ? launch_count<EJ_TABLE_HASH, true>(h, pp, P, t, wcount)
                   : launch_count<EJ_TABLE_HASH, false>(h, pp, P, t, wcount));
    else
      EJ_TRY(outer ? launch_count<EJ_TABLE_SORTED, true>(h, pp, P, t, wcount)
                   : launch_count<EJ_TABLE_SORTED, false>(h, pp, P, t, wcount));
  }
  EJ_TRY(ej_scan_u64_u64(h, wcount, pp.nwtiles, woff, ej_arena_at(h, pp.scan_off)));
  if (d_count)
    EJ_CUDA(h, cudaMemcpyAsync(d_count, woff + pp.nwtiles, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                               h->stream));
  return EJ_OK;
}

ej_status ej_probe_write(ej_handle* h, const ej_probe_plan_t& pp, const ej_tuple* P, const ej_table_view& t,
                         bool outer, ej_result* out, uint64_t cap, unsigned long long* d_count) {
  if (!pp.ntiles) {
    EJ_CUDA(h, cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), h->stream));
    return EJ_OK;
  }
  if (t.kind == EJ_TABLE_HASH)
    return outer ? launch_write<EJ_TABLE_HASH, true>(h, pp, P, t, out, cap, d_count)
                 : launch_write<EJ_TABLE_HASH, false>(h, pp, P, t, out, cap, d_count);
  return outer ? launch_write<EJ_TABLE_SORTED, true>(h, pp, P, t, out, cap, d_count)
               : launch_write<EJ_TABLE_SORTED, false>(h, pp, P, t, out, cap, d_count);
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

// Partition S (when the layout says so), then either count (+ scan) or write
// with look-back; records phase marks 2..4 (the caller has begun the set and
// marked the build).  The arena must already hold the layout, reserved
// together with anything the table placed there, so that no reservation
// moves a built table.
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
  if (count_only) {
    EJ_TRY(ej_probe_count(h, L.pp, P, t, outer, d_count));
    ej_phase_mark(h, 3);
  } else {
    ej_phase_mark(h, 3);
    EJ_TRY(ej_probe_write(h, L.pp, P, t, outer, out, out_cap, d_count));
  }
  ej_phase_mark(h, 4);
  return EJ_OK;
}

ej_status ej_hash_join_run(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                           ej_result* out, uint64_t out_cap, unsigned long long* d_count, int mode) {
  // mode: 0 = partition S when the planner says so, 1 = never partition S, 2 = count only
  const uint32_t pb = (mode == 1) ? 0u : ej_probe_partition_bits(h, nR, nS);
  ej_plan_bytes p;
  ej_table_plan_t tp;
  ej_table_plan(p, tp, nR, /*own_storage=*/false, EJ_TABLE_HASH, ej_tuned_bucket_delta(h, nR));
  ej_probe_layout L;
  ej_probe_layout_add(p, L, nS, pb);
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  ej_phase_begin(h);
  ej_table_view t;
  EJ_TRY(ej_table_build(h, tp, R, reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rkey_off)),
                        reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rval_off)), ej_arena_at(h, tp.aux_off), &t));
  ej_phase_mark(h, 1);
  return ej_probe_exec(h, L, t, S, /*outer=*/false, mode == 2, out, out_cap, d_count);
}
