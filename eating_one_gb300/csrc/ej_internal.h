// ej_internal.h - host-side internals shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "ej.h"

// Bounded device waits (decoupled look-back, mbarrier waits) give up after
// this many nanoseconds unless the handle sets another limit
// (EJ_OPT_WAIT_LIMIT_NS); a kernel draining its own copies in flight after
// giving up always allows this long.
constexpr unsigned long long EJ_DEFAULT_WAIT_LIMIT_NS = 1000000000ull;

// Device status word: the first error a kernel records wins (atomicCAS on code).
struct ej_dev_status {
  unsigned int code;  // ej_status
  unsigned int info;  // kernel-specific detail (e.g. which wait gave up)
  unsigned long long aux;
};

// the table, partitioned probe side and run descriptors that a hash-join
// count leaves for the write of the same join (hash_join.cu)
struct ej_prepared_join;

struct ej_zipf_cache {
  double s = -1.0;
  uint32_t domain = 0;
  double* d_cdf = nullptr;
};

struct ej_handle {
  int device = 0;
  int num_sms = 0;
  size_t l2_bytes = 0;
  cudaStream_t stream = nullptr;
  // scratch arena (bump allocation, reset per call)
  void* arena = nullptr;
  size_t arena_cap = 0;
  size_t arena_peak = 0;
  // small device words
  ej_dev_status* d_status = nullptr;
  unsigned long long* d_words = nullptr;  // [0] = join count, [1..7] scratch
  unsigned long long* h_words = nullptr;  // pinned host mirror
  ej_dev_status* h_status = nullptr;      // pinned host mirror of d_status
  std::string last_error;
  // phase timing: a ring of EJ_PHASE_RING sets of EJ_PHASES+1 events
  bool timing = false;
  std::vector<cudaEvent_t> ring;
  uint32_t ring_head = 0;     // next set to record
  uint32_t ring_pending = 0;  // recorded sets not yet summed by ej_phase_totals
  int cur_set = -1;           // set of the join being recorded, -1 when none
  int last_set = -1;          // last fully recorded set
  unsigned long long launches = 0;  // kernels launched through ej_check_launch
  ej_zipf_cache zipf;
  // tuning overrides (-1 / 0 = planner's choice) and the autotuned table
  int opt_partition_bits = -1;
  int opt_bucket_delta = 0;
  bool opt_bucket_delta_set = false;
  int opt_build = 0;        // EJ_BUILD_* (0: tuning table, then planner)
  int opt_table = 0;        // EJ_TABLE_FORMAT_*
  int opt_probe_warps = 0;  // 4 or 8 (0: tuning table, then 8)
  std::vector<ej_tune_entry> tuning;  // ascending log2_rows
  // host-buffer entry points: device staging owned separately from the arena
  void* stage = nullptr;
  size_t stage_cap = 0;
  // chunked host-buffer joins: copy streams, events, device and pinned buffers
  struct ej_stream_res* sres = nullptr;
  // synchronous batched joins: per-join counts
  unsigned long long* d_batch_counts = nullptr;
  unsigned long long* h_batch_counts = nullptr;
  uint32_t batch_counts_cap = 0;
  // a hash-join count kept for the write that follows it (ej_hash_join_count
  // then ej_hash_join on the same relations); any other use of the arena
  // drops it (ej_arena_reserve)
  ej_prepared_join* prep = nullptr;
  bool prep_valid = false;
  bool opt_count_reuse = true;
  // bound of every device-side wait of this handle's kernels (EJ_OPT_WAIT_LIMIT_NS)
  unsigned long long wait_limit_ns = EJ_DEFAULT_WAIT_LIMIT_NS;
};

// Arena layout: callers first add every buffer to a plan, then reserve once.
struct ej_plan_bytes {
  size_t bytes = 0;
  size_t add(size_t n) {
    size_t off = bytes;
    bytes += (n + 255) & ~size_t(255);
    return off;
  }
};

// Every device and pinned-host allocation of the library goes through these,
// so that ej_inject_alloc_failures can make them fail (api.cu).
bool ej_alloc_failure_injected();
template <class T>
inline cudaError_t ej_dev_alloc(T** p, size_t bytes) {
  if (ej_alloc_failure_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}
template <class T>
inline cudaError_t ej_host_alloc(T** p, size_t bytes) {
  if (ej_alloc_failure_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost(reinterpret_cast<void**>(p), bytes);
}
template <class T>
inline cudaError_t ej_pool_alloc(T** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s) {
  if (ej_alloc_failure_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, pool, s);
}

ej_status ej_fail(ej_handle* h, ej_status s, const char* fmt, ...);
// on the handle's stream: d_sums[i] = ej_checksum of the first
// min(d_counts[i], d_desc[i].out_cap) rows of d_desc[i].out, i < n (device arrays)
ej_status ej_checksum_outputs_async(ej_handle* h, const ej_join_desc* d_desc, const unsigned long long* d_counts,
                                    uint32_t n, unsigned long long* d_sums);
// frees the chunked-join resources (stream_join.cu); safe on a handle without them
void ej_stream_release(ej_handle* h);
// block nested loop over R x S (bnlj.cu); rows go to out at positions taken
// from *cursor, which is not reset, so successive calls append
ej_status ej_bnl_append(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                        ej_result* out, uint64_t cap, unsigned long long* cursor);
ej_status ej_arena_reserve(ej_handle* h, size_t bytes);
inline char* ej_arena_at(ej_handle* h, size_t off) { return static_cast<char*>(h->arena) + off; }
ej_status ej_check_launch(ej_handle* h, const char* what);
// the index memory pool of a device gives back the memory no index holds (index.cu)
void ej_index_pool_trim(int device);
// phase timing: begin a join's event set (mark 0), then marks 1..EJ_PHASES at
// the phase boundaries (build | partition | count | write); no-ops when timing is off
void ej_phase_begin(ej_handle* h);
void ej_phase_mark(ej_handle* h, int k);

#define EJ_CUDA(h, call)                                                                  \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return ej_fail((h), EJ_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                     __FILE__, __LINE__);                                                 \
  } while (0)

#define EJ_TRY(...)                  \
  do {                               \
    ej_status s_ = (__VA_ARGS__);    \
    if (s_ != EJ_OK) return s_;      \
  } while (0)

static inline uint32_t ej_ceil_log2(uint64_t x) {
  uint32_t b = 0;
  while ((uint64_t(1) << b) < x) b++;
  return b;
}

// ---- prefix scan (scan.cu) ----------------------------------------------
// Exclusive scan of n inputs into n+1 outputs (out[n] = total).  `scratch`
// must hold ej_scan_scratch_bytes(n) bytes of device memory.
size_t ej_scan_scratch_bytes(uint64_t n);
ej_status ej_scan_u32_u32(ej_handle* h, const uint32_t* in, uint64_t n, uint32_t* out, void* scratch);
ej_status ej_scan_u32_u64(ej_handle* h, const uint32_t* in, uint64_t n, unsigned long long* out,
                          void* scratch);
ej_status ej_scan_u64_u64(ej_handle* h, const unsigned long long* in, uint64_t n,
                          unsigned long long* out, void* scratch);

// ---- radix partitioning (radix.cu) ---------------------------------------
// Stable partition of tuples by digit = (key(val) >> shift) & ((1<<bits)-1),
// key = hash32(val) (EJ_DIGIT_HASH) or the order-preserving unsigned image of
// the signed val (EJ_DIGIT_VALUE, for sorting).
enum { EJ_DIGIT_HASH = 0, EJ_DIGIT_VALUE = 1 };
constexpr uint32_t EJ_RX_TILE = 4096;  // rows per radix tile
// A tile of a segmented pass (batched joins): rows [start, start + n) of one
// segment (n <= EJ_RX_TILE); the histogram cell of digit d is cell0 + d * stride,
// with cells laid out segment by segment (cell0 = segment base + tile index
// in the segment, stride = tiles of the segment), so one scan over all cells
// keeps the segments apart in the output.
struct ej_rx_tile {
  unsigned long long start;
  uint32_t n, cell0, stride, pad;
  const ej_tuple* src;  // the tile's first input row (ej_partition_pass_src; other passes: input + start)
};

struct ej_radix_plan {
  uint64_t n = 0;
  uint32_t ntiles = 0;
  size_t hist_off = 0, offs_off = 0, scan_off = 0;  // arena offsets
  const ej_rx_tile* tiles = nullptr;                // device descriptors (segmented passes)
};
uint32_t ej_radix_tiles(uint64_t n);
void ej_radix_plan_add(ej_plan_bytes& p, ej_radix_plan& rp, uint64_t n);
ej_status ej_radix_pass(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, ej_tuple* out,
                        uint32_t shift, uint32_t bits, int digit_kind = EJ_DIGIT_HASH);
// the same pass writing keys and vals to two arrays (last pass of a table build)
// a pass whose order within a digit is unspecified: a one-pass partition, or
// the first pass of an LSD sort (the later, stable passes decide every order
// that matters)
ej_status ej_partition_pass(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, ej_tuple* out,
                            uint32_t shift, uint32_t bits, int digit_kind = EJ_DIGIT_HASH);
ej_status ej_radix_pass_soa(ej_handle* h, const ej_radix_plan& rp, const ej_tuple* in, int32_t* out_keys,
                            int32_t* out_vals, uint32_t shift, uint32_t bits, int digit_kind);
// the unordered pass by hash digits over tiles whose descriptors carry their
// source rows (src), which may lie in separate arrays
ej_status ej_partition_pass_src(ej_handle* h, const ej_radix_plan& rp, ej_tuple* out, uint32_t shift,
                                uint32_t bits);

// ---- probe targets (hash_join.cu) -----------------------------------------
// R is stored as two arrays, rkey[] and rval[], in one order:
// EJ_TABLE_HASH: sorted by hash32(val), so equal keys form one contiguous run
//   and bucket b (top `hb` hash bits) is rows [bucket[b].x, bucket[b].y)
//   (both bounds in one 8-byte word, so a probe reads them with one load).
// EJ_TABLE_SORTED: sorted by val; bucket b of value v = (v - vmin) >> vshift
//   is rows [bucket[b].x, bucket[b].y), with vmin, vmax and vshift in a
//   16-byte device header (vbuckets) written after the sort.
// Both arrays carry EJ_TABLE_PAD readable elements past nR (vector loads).
enum { EJ_TABLE_HASH = 0, EJ_TABLE_SORTED = 1 };
constexpr uint64_t EJ_TABLE_PAD = 8;
struct ej_table_view {
  int kind = EJ_TABLE_HASH;
  const int32_t* rkey = nullptr;     // [nR + pad] row ids in table order
  const int32_t* rval = nullptr;     // [nR + pad] join keys in table order
  const uint2* bucket = nullptr;     // [2^hb] (hash, batched tables): row bounds of each bucket
  const uint2* dir = nullptr;        // (hash, single tables) key directory {hash, run start [, length]}
  const uint32_t* dir_bits = nullptr;  // device word: the directory has 2^bits home slots
  uint32_t dir_packed = 0;             // entries {hash, start << 5 | run length} (tables under 2^27 rows)
  const void* vbuckets = nullptr;    // (sorted) device EjValueBuckets {vmin, vmax, vshift} of `bucket`
  uint64_t nR = 0;
  uint32_t hb = 1;
  uint32_t voff = 0;  // rval - voff is 16-byte aligned (tables of a batch share one array)
  // known on the host to have runs of about one row (an index whose build
  // chose bucket bounds for its short runs): probes load run keys in 8-byte chunks
  uint32_t short_runs = 0;
};
uint32_t ej_table_bucket_bits(uint64_t nR, int delta = 0);
// the bucket-bits delta and the S partition bits (-1: planner) that apply to a
// build side of nR rows: explicit options first, then the tuning table
int ej_tuned_bucket_delta(const ej_handle* h, uint64_t nR, int planner = 0);
int ej_tuned_partition_bits(const ej_handle* h, uint64_t nR);
// the build's radix passes, the table format (0: planner) and the probe
// kernels' warps per block that apply to a build side of nR rows
int ej_tuned_build(const ej_handle* h, uint64_t nR);
int ej_tuned_table_format(const ej_handle* h, uint64_t nR);
int ej_tuned_probe_warps(const ej_handle* h, uint64_t nR);
