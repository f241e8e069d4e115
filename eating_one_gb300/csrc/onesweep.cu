// onesweep.cu - LSD radix sort of a table's rows in one scatter launch per
// digit (Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix
// Sort for GPUs", 2022, restated).
//
// The LSD build of radix.cu spends three launches per 8-bit digit: a
// histogram pass reading the whole input, a scan of the digit-major
// histogram, and the scatter.  Here:
//   1. one pass reads the input once and counts all four digits of every
//      row's order key (per-block shared-memory counters, one global atomic
//      per counter and block);
//   2. one block turns the four 256-entry histograms into each digit's global
//      base;
//   3. per digit, one scatter launch: tiles take ids in launch order from an
//      atomic counter, rank their 4096 rows stably (the ballot ranking of
//      radix.cu), publish each digit's count, and learn the counts of the
//      tiles before them by a decoupled look-back per digit (thread d walks
//      back over digit d's status words) instead of from a scan; the last
//      pass writes the table's two columns.
// Status words pack a 2-bit flag (aggregate / inclusive prefix) over a 62-bit
// count.  Waits are bounded by the handle's wait limit; a wait that runs out
// takes the missing counts as zero (positions then come out too small, never
// too large, so every store stays inside the output) and reports
// EJ_ERR_TIMEOUT.
//
// Replaces, for the sort index, the reference's CPU quicksort of BUCKET{val,
// adr} (joins/innerJoin_gpu/sort_index/main_street/inner-idx-bnlj.cc:175-217).
#include "ej_device.cuh"
#include "onesweep.cuh"

namespace {

constexpr int OS_THREADS = 256;
constexpr int OS_WARPS = OS_THREADS / 32;
constexpr int OS_TILE = (int)EJ_RX_TILE;          // rows per tile
constexpr int OS_WARP_SPAN = OS_TILE / OS_WARPS;  // consecutive rows per warp
constexpr int OS_ROUNDS = OS_WARP_SPAN / 32;
constexpr int OS_DIGITS = 256;
constexpr int OS_PASSES = 4;

template <int KIND>
__device__ __forceinline__ uint32_t os_key(int32_t val) {
  return KIND == EJ_DIGIT_HASH ? ej_hash32((uint32_t)val) : ((uint32_t)val ^ 0x80000000u);
}

// all four digit histograms: hist[p * 256 + d] (zeroed by the caller)
template <int KIND>
__global__ void __launch_bounds__(OS_THREADS) os_hist_kernel(const ej_tuple* __restrict__ in, uint64_t n,
                                                              uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[OS_PASSES * OS_DIGITS];
  for (int i = threadIdx.x; i < OS_PASSES * OS_DIGITS; i += OS_THREADS) cnt[i] = 0u;
  __syncthreads();
  const int* vals = reinterpret_cast<const int*>(in) + 1;
  for (uint64_t i = (uint64_t)blockIdx.x * OS_THREADS + threadIdx.x; i < n; i += (uint64_t)gridDim.x * OS_THREADS) {
    const uint32_t k = os_key<KIND>(__ldcs(vals + 2 * i));
#pragma unroll
    for (int p = 0; p < OS_PASSES; p++) atomicAdd(&cnt[p * OS_DIGITS + ((k >> (8 * p)) & 255u)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < OS_PASSES * OS_DIGITS; i += OS_THREADS)
    if (cnt[i]) atomicAdd(&hist[i], cnt[i]);
}

// each pass's digit bases: base[p * 256 + d] = rows of pass p's digits below d
__global__ void __launch_bounds__(OS_DIGITS) os_base_kernel(const uint32_t* __restrict__ hist,
                                                            uint32_t* __restrict__ base) {
  __shared__ uint32_t tmp[OS_DIGITS / 32 + 1];
  for (int p = 0; p < OS_PASSES; p++) {
    uint32_t total;
    const uint32_t ex = ej_block_exclusive_sum<OS_DIGITS, uint32_t>(hist[p * OS_DIGITS + threadIdx.x], tmp, &total);
    base[p * OS_DIGITS + threadIdx.x] = ex;
  }
}

struct OsSmem {
  ej_tuple sorted[OS_TILE];              // 32 KB: the tile in digit order
  uint32_t cnt[OS_WARPS][OS_DIGITS];     // per-warp digit counters, then tile positions
  uint32_t gbase[OS_DIGITS];
  uint32_t warp_tmp[OS_WARPS + 1];
  uint32_t tile;
};

#define OS_FLAG_AGG 1ull
#define OS_FLAG_PREFIX 2ull
#define OS_VALUE_MASK ((1ull << 62) - 1ull)

// One digit pass.  status[tile * 256 + d] (zeroed by the caller) carries the
// tiles' digit counts; *tile_ctr hands out tile ids in launch order.
template <int KIND, bool SOA>
__global__ void __launch_bounds__(OS_THREADS, 4)
os_scatter_kernel(const ej_tuple* __restrict__ in, uint64_t n, ej_tuple* __restrict__ out, int32_t* __restrict__ out_keys,
                  int32_t* __restrict__ out_vals, const uint32_t* __restrict__ base, unsigned long long* status,
                  unsigned int* tile_ctr, uint32_t shift, ej_dev_status* st, unsigned long long wait_ns) {
  extern __shared__ __align__(16) unsigned char os_smem_raw[];
  OsSmem& sm = *reinterpret_cast<OsSmem*>(os_smem_raw);
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < OS_WARPS * OS_DIGITS; i += OS_THREADS) (&sm.cnt[0][0])[i] = 0u;
  if (threadIdx.x == 0) sm.tile = atomicAdd(tile_ctr, 1u);
  __syncthreads();
  const uint64_t tile = sm.tile;
  const uint64_t start = tile * OS_TILE;
  const uint32_t tile_n = (uint32_t)min((uint64_t)OS_TILE, n - start);

  // 1. the warp's consecutive rows into registers (coalesced, streaming)
  const uint32_t wbase = warp * OS_WARP_SPAN;
  const uint2* src = reinterpret_cast<const uint2*>(in + start);
  uint2 tup[OS_ROUNDS];
#pragma unroll
  for (int r = 0; r < OS_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    tup[r] = i < tile_n ? __ldcs(src + i) : make_uint2(0u, 0u);
  }

  // 2. stable rank within the warp (round order, then lane order): the lanes
  //    sharing a digit from one ballot per digit bit, the warp's running
  //    count of each digit in its shared-memory counter
  uint32_t packed[OS_ROUNDS];
#pragma unroll
  for (int r = 0; r < OS_ROUNDS; r++) {
    const uint32_t i = wbase + r * 32u + lane;
    const bool valid = i < tile_n;
    const uint32_t d = valid ? (os_key<KIND>((int32_t)tup[r].y) >> shift) & 255u : 0u;
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

  // 3. thread d: the tile's count of digit d, published at once; warp bases
  //    within the digit; the digit's start in the tile
  const uint32_t d = threadIdx.x;
  uint32_t total = 0;
#pragma unroll
  for (int w = 0; w < OS_WARPS; w++) {
    const uint32_t c = sm.cnt[w][d];
    sm.cnt[w][d] = total;
    total += c;
  }
  unsigned long long* my = status + tile * OS_DIGITS + d;
  ej_st_relaxed(my, ((tile == 0 ? OS_FLAG_PREFIX : OS_FLAG_AGG) << 62) | total);
  uint32_t all;
  const uint32_t dstart = ej_block_exclusive_sum<OS_THREADS, uint32_t>(total, sm.warp_tmp, &all);
#pragma unroll
  for (int w = 0; w < OS_WARPS; w++) sm.cnt[w][d] += dstart;

  // 4. decoupled look-back of digit d over the tiles before this one
  unsigned long long excl = 0;
  if (tile > 0) {
    const unsigned long long t0 = ej_globaltimer();
    const unsigned int period = wait_ns < 100000ull ? 0u : 63u;
    bool gave_up = false;
    for (int64_t k = (int64_t)tile - 1; k >= 0; k--) {
      unsigned long long w = ej_ld_relaxed(status + (uint64_t)k * OS_DIGITS + d);
      for (unsigned int spins = 1; (w >> 62) == 0ull && !gave_up; spins++) {
        __nanosleep(spins < 8 ? 32u : 256u);
        w = ej_ld_relaxed(status + (uint64_t)k * OS_DIGITS + d);
        if ((spins & period) == 0u && ej_globaltimer() - t0 >= wait_ns) gave_up = true;
      }
      excl += w & OS_VALUE_MASK;  // a tile given up on counts as zero
      if ((w >> 62) == OS_FLAG_PREFIX || gave_up) break;
    }
    ej_st_relaxed(my, (OS_FLAG_PREFIX << 62) | ((excl + total) & OS_VALUE_MASK));
    if (gave_up) ej_set_status(st, EJ_ERR_TIMEOUT, 3u);
  }
  sm.gbase[d] = base[d] + (uint32_t)excl - dstart;
  __syncthreads();

  // 5. every row to its place in the tile's digit order (shared memory)
#pragma unroll
  for (int r = 0; r < OS_ROUNDS; r++)
    if (packed[r] != 0xFFFFFFFFu)
      reinterpret_cast<uint2*>(sm.sorted)[sm.cnt[warp][packed[r] >> 16] + (packed[r] & 0xFFFFu)] = tup[r];
  __syncthreads();

  // 6. digit runs out: sorted position k goes to gbase[digit] + k
  for (uint32_t k = threadIdx.x; k < tile_n; k += OS_THREADS) {
    const uint2 t = reinterpret_cast<const uint2*>(sm.sorted)[k];
    const uint32_t pos = sm.gbase[(os_key<KIND>((int32_t)t.y) >> shift) & 255u] + k;
    if (SOA) {
      out_keys[pos] = (int32_t)t.x;
      out_vals[pos] = (int32_t)t.y;
    } else {
      reinterpret_cast<uint2*>(out)[pos] = t;
    }
  }
}

template <int KIND>
ej_status os_sort_kind(ej_handle* h, const ej_onesweep_plan& op, const ej_tuple* R, ej_tuple* tmp_a, ej_tuple* tmp_b,
                       int32_t* rkey, int32_t* rval) {
  uint32_t* hist = reinterpret_cast<uint32_t*>(ej_arena_at(h, op.hist_off));
  uint32_t* base = reinterpret_cast<uint32_t*>(ej_arena_at(h, op.base_off));
  unsigned long long* status = reinterpret_cast<unsigned long long*>(ej_arena_at(h, op.status_off));
  unsigned int* ctr = reinterpret_cast<unsigned int*>(ej_arena_at(h, op.ctr_off));
  EJ_CUDA(h, cudaMemsetAsync(hist, 0, OS_PASSES * OS_DIGITS * sizeof(uint32_t), h->stream));
  const unsigned hblocks = (unsigned)std::min<uint64_t>((op.n + OS_THREADS * 16 - 1) / (OS_THREADS * 16),
                                                        (uint64_t)h->num_sms * 8);
  os_hist_kernel<KIND><<<hblocks, OS_THREADS, 0, h->stream>>>(R, op.n, hist);
  EJ_TRY(ej_check_launch(h, "os_hist_kernel"));
  os_base_kernel<<<1, OS_DIGITS, 0, h->stream>>>(hist, base);
  EJ_TRY(ej_check_launch(h, "os_base_kernel"));
  EJ_CUDA(h, cudaFuncSetAttribute(os_scatter_kernel<KIND, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(OsSmem)));
  EJ_CUDA(h, cudaFuncSetAttribute(os_scatter_kernel<KIND, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(OsSmem)));
  const ej_tuple* src = R;
  ej_tuple* dst[2] = {tmp_a, tmp_b};
  for (int p = 0; p < OS_PASSES; p++) {
    EJ_CUDA(h, cudaMemsetAsync(status, 0, op.status_bytes, h->stream));
    EJ_CUDA(h, cudaMemsetAsync(ctr, 0, sizeof(unsigned int), h->stream));
    if (p + 1 == OS_PASSES) {
      os_scatter_kernel<KIND, true><<<op.ntiles, OS_THREADS, sizeof(OsSmem), h->stream>>>(
          src, op.n, nullptr, rkey, rval, base + p * OS_DIGITS, status, ctr, 8u * p, h->d_status, h->wait_limit_ns);
    } else {
      os_scatter_kernel<KIND, false><<<op.ntiles, OS_THREADS, sizeof(OsSmem), h->stream>>>(
          src, op.n, dst[p & 1], nullptr, nullptr, base + p * OS_DIGITS, status, ctr, 8u * p, h->d_status,
          h->wait_limit_ns);
      src = dst[p & 1];
    }
    EJ_TRY(ej_check_launch(h, "os_scatter_kernel"));
  }
  return EJ_OK;
}

}  // namespace

void ej_onesweep_plan_add(ej_plan_bytes& p, ej_onesweep_plan& op, uint64_t n) {
  op.n = n;
  op.ntiles = (uint32_t)((n + OS_TILE - 1) / OS_TILE);
  op.hist_off = p.add(OS_PASSES * OS_DIGITS * sizeof(uint32_t));
  op.base_off = p.add(OS_PASSES * OS_DIGITS * sizeof(uint32_t));
  op.status_bytes = (size_t)(op.ntiles ? op.ntiles : 1) * OS_DIGITS * sizeof(unsigned long long);
  op.status_off = p.add(op.status_bytes);
  op.ctr_off = p.add(sizeof(unsigned int));
}

ej_status ej_onesweep_sort(ej_handle* h, const ej_onesweep_plan& op, const ej_tuple* R, ej_tuple* tmp_a,
                           ej_tuple* tmp_b, int32_t* rkey, int32_t* rval, int digit_kind) {
  if (op.n == 0) return EJ_OK;
  if (op.n >= 0xFFFFFFFFull) return ej_fail(h, EJ_ERR_TOO_LARGE, "table of %llu rows", (unsigned long long)op.n);
  return digit_kind == EJ_DIGIT_VALUE ? os_sort_kind<EJ_DIGIT_VALUE>(h, op, R, tmp_a, tmp_b, rkey, rval)
                                      : os_sort_kind<EJ_DIGIT_HASH>(h, op, R, tmp_a, tmp_b, rkey, rval);
}
