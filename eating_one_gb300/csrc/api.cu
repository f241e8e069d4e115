// api.cu - C ABI entry points: handle, arena, status plumbing, hash joins,
// generators, checksum, scan and the host-buffer path.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "ej_device.cuh"
#include "hash_join.cuh"
#include "ej_entry.h"

// ---- allocation-failure injection (tests) ----------------------------------

static std::atomic<uint32_t> g_alloc_failures{0};

extern "C" void ej_inject_alloc_failures(uint32_t count) { g_alloc_failures.store(count); }

bool ej_alloc_failure_injected() {
  uint32_t c = g_alloc_failures.load(std::memory_order_relaxed);
  while (c > 0)
    if (g_alloc_failures.compare_exchange_weak(c, c - 1)) return true;
  return false;
}

// ---- errors ---------------------------------------------------------------

ej_status ej_fail(ej_handle* h, ej_status s, const char* fmt, ...) {
  if (h) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->last_error = buf;
  }
  return s;
}

ej_status ej_check_launch(ej_handle* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ej_fail(h, EJ_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
  h->launches++;
  return EJ_OK;
}

extern "C" const char* ej_status_name(ej_status s) {
  switch (s) {
    case EJ_OK: return "EJ_OK";
    case EJ_ERR_INVALID: return "EJ_ERR_INVALID";
    case EJ_ERR_CAPACITY: return "EJ_ERR_CAPACITY";
    case EJ_ERR_CUDA: return "EJ_ERR_CUDA";
    case EJ_ERR_NOMEM: return "EJ_ERR_NOMEM";
    case EJ_ERR_TIMEOUT: return "EJ_ERR_TIMEOUT";
    case EJ_ERR_TOO_LARGE: return "EJ_ERR_TOO_LARGE";
    case EJ_ERR_NO_DEVICE: return "EJ_ERR_NO_DEVICE";
    case EJ_ERR_BUSY: return "EJ_ERR_BUSY";
    case EJ_ERR_INTERNAL: return "EJ_ERR_INTERNAL";
    case EJ_ERR_IO: return "EJ_ERR_IO";
  }
  return "EJ_ERR_UNKNOWN";
}

extern "C" const char* ej_last_error(const ej_handle* h) { return h ? h->last_error.c_str() : ""; }

// ---- handle -------------------------------------------------------------

extern "C" ej_status ej_create(int device, ej_handle** out) {
  if (!out) return EJ_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return EJ_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return EJ_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return EJ_ERR_CUDA;
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  if (major != 10 || minor != 3) return EJ_ERR_NO_DEVICE;  // built for sm_103a only
  ej_handle* h = new ej_handle();
  h->device = device;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
  int l2 = 0;
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
  h->l2_bytes = (size_t)l2;
  bool ok = ej_dev_alloc(&h->d_status, sizeof(ej_dev_status)) == cudaSuccess &&
            ej_dev_alloc(&h->d_words, 8 * sizeof(unsigned long long)) == cudaSuccess &&
            ej_host_alloc(&h->h_words, 8 * sizeof(unsigned long long)) == cudaSuccess &&
            ej_host_alloc(&h->h_status, sizeof(ej_dev_status)) == cudaSuccess;
  if (ok) ok = cudaMemset(h->d_status, 0, sizeof(ej_dev_status)) == cudaSuccess &&
               cudaMemset(h->d_words, 0, 8 * sizeof(unsigned long long)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    ej_destroy(h);
    return EJ_ERR_NOMEM;
  }
  *out = h;
  return EJ_OK;
}

extern "C" ej_status ej_destroy(ej_handle* h) {
  if (!h) return EJ_ERR_INVALID;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  ej_stream_release(h);
  cudaFree(h->arena);
  cudaFree(h->stage);
  cudaFree(h->d_status);
  cudaFree(h->d_words);
  cudaFree(h->zipf.d_cdf);
  cudaFreeHost(h->h_words);
  cudaFreeHost(h->h_status);
  cudaFree(h->d_batch_counts);
  cudaFreeHost(h->h_batch_counts);
  for (cudaEvent_t e : h->ring) cudaEventDestroy(e);
  delete h->prep;
  delete h;
  return EJ_OK;
}

extern "C" ej_status ej_set_stream(ej_handle* h, ej_stream stream) {
  if (!h) return EJ_ERR_INVALID;
  h->stream = static_cast<cudaStream_t>(stream);
  return EJ_OK;
}

extern "C" uint64_t ej_scratch_bytes(const ej_handle* h) { return h ? (uint64_t)h->arena_cap : 0; }

extern "C" ej_status ej_trim(ej_handle* h) {
  if (!h) return EJ_ERR_INVALID;
  EJ_CUDA(h, cudaSetDevice(h->device));
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  ej_stream_release(h);
  h->prep_valid = false;
  EJ_CUDA(h, cudaFree(h->arena));
  EJ_CUDA(h, cudaFree(h->stage));
  h->arena = h->stage = nullptr;
  h->arena_cap = h->stage_cap = 0;
  ej_index_pool_trim(h->device);
  return EJ_OK;
}

extern "C" ej_status ej_set_timing(ej_handle* h, int enable) {
  if (!h) return EJ_ERR_INVALID;
  if (enable && h->ring.empty()) {
    EJ_CUDA(h, cudaSetDevice(h->device));
    h->ring.resize((size_t)EJ_PHASE_RING * (EJ_PHASES + 1), nullptr);
    for (cudaEvent_t& e : h->ring) EJ_CUDA(h, cudaEventCreate(&e));
  }
  h->timing = enable != 0;
  return EJ_OK;
}

extern "C" uint64_t ej_kernel_launches(const ej_handle* h) { return h ? (uint64_t)h->launches : 0; }

void ej_phase_begin(ej_handle* h) {
  if (!h->timing || h->ring.empty()) {
    h->cur_set = -1;
    return;
  }
  h->cur_set = (int)h->ring_head;
  h->ring_head = (h->ring_head + 1) % EJ_PHASE_RING;
  cudaEventRecord(h->ring[(size_t)h->cur_set * (EJ_PHASES + 1)], h->stream);
}

void ej_phase_mark(ej_handle* h, int k) {
  if (h->cur_set < 0) return;
  cudaEventRecord(h->ring[(size_t)h->cur_set * (EJ_PHASES + 1) + k], h->stream);
  if (k == EJ_PHASES) {
    h->last_set = h->cur_set;
    h->cur_set = -1;
    if (h->ring_pending < EJ_PHASE_RING) h->ring_pending++;
  }
}

static ej_status set_phases(ej_handle* h, int set, float ms[EJ_PHASES]) {
  cudaEvent_t* e = &h->ring[(size_t)set * (EJ_PHASES + 1)];
  EJ_CUDA(h, cudaEventSynchronize(e[EJ_PHASES]));
  for (int i = 0; i < EJ_PHASES; i++) EJ_CUDA(h, cudaEventElapsedTime(&ms[i], e[i], e[i + 1]));
  return EJ_OK;
}

extern "C" ej_status ej_set_option(ej_handle* h, ej_option opt, int64_t value) {
  if (!h) return EJ_ERR_INVALID;
  switch (opt) {
    case EJ_OPT_PROBE_PARTITION_BITS:
      if (value < -1 || value > 8) return ej_fail(h, EJ_ERR_INVALID, "partition bits must be -1..8");
      h->opt_partition_bits = (int)value;
      return EJ_OK;
    case EJ_OPT_BUCKET_BITS_DELTA:
      if (value < -3 || value > 3) return ej_fail(h, EJ_ERR_INVALID, "bucket bits delta must be -3..3");
      h->opt_bucket_delta = (int)value;
      h->opt_bucket_delta_set = value != 0;  // 0 hands the choice back to the tuning table
      return EJ_OK;
    case EJ_OPT_WAIT_LIMIT_NS:
      if (value < -1 || value > 10000000000ll) return ej_fail(h, EJ_ERR_INVALID, "wait limit must be -1..1e10 ns");
      h->wait_limit_ns = value < 0 ? EJ_DEFAULT_WAIT_LIMIT_NS : (unsigned long long)value;
      return EJ_OK;
    case EJ_OPT_BUILD:
      if (value < EJ_BUILD_PLANNER || value > EJ_BUILD_ONESWEEP) return ej_fail(h, EJ_ERR_INVALID, "build must be 0..3");
      h->opt_build = (int)value;
      return EJ_OK;
    case EJ_OPT_TABLE:
      if (value < EJ_TABLE_FORMAT_PLANNER || value > EJ_TABLE_FORMAT_DIRECTORY)
        return ej_fail(h, EJ_ERR_INVALID, "table format must be 0..2");
      h->opt_table = (int)value;
      return EJ_OK;
    case EJ_OPT_PROBE_WARPS:
      if (value != 0 && value != 4 && value != 8) return ej_fail(h, EJ_ERR_INVALID, "probe warps must be 0, 4 or 8");
      h->opt_probe_warps = (int)value;
      return EJ_OK;
    case EJ_OPT_COUNT_REUSE:
      if (value != 0 && value != 1) return ej_fail(h, EJ_ERR_INVALID, "count reuse is 0 or 1");
      h->opt_count_reuse = value != 0;
      if (!h->opt_count_reuse) h->prep_valid = false;
      return EJ_OK;
  }
  return ej_fail(h, EJ_ERR_INVALID, "unknown option %d", (int)opt);
}

extern "C" ej_status ej_set_tuning(ej_handle* h, const ej_tune_entry* entries, uint32_t n) {
  if (!h || (n && !entries)) return EJ_ERR_INVALID;
  std::vector<ej_tune_entry> t(entries, entries + n);
  for (const ej_tune_entry& e : t) {
    if (e.log2_rows > 32 || e.partition_bits < -1 || e.partition_bits > 8 || e.bucket_delta < -3 ||
        e.bucket_delta > 3 || e.build < EJ_BUILD_PLANNER || e.build > EJ_BUILD_ONESWEEP ||
        e.table < EJ_TABLE_FORMAT_PLANNER || e.table > EJ_TABLE_FORMAT_DIRECTORY ||
        (e.probe_warps != 0 && e.probe_warps != 4 && e.probe_warps != 8))
      return ej_fail(h, EJ_ERR_INVALID, "bad tuning entry (log2_rows %u)", e.log2_rows);
  }
  std::sort(t.begin(), t.end(),
            [](const ej_tune_entry& a, const ej_tune_entry& b) { return a.log2_rows < b.log2_rows; });
  h->tuning = t;
  return EJ_OK;
}

static const ej_tune_entry* tuning_for(const ej_handle* h, uint64_t nR) {
  const ej_tune_entry* best = nullptr;
  const uint32_t lg = ej_ceil_log2(nR < 1 ? 1 : nR);
  for (const ej_tune_entry& e : h->tuning)
    if (e.log2_rows <= lg) best = &e;
  return best;
}

int ej_tuned_bucket_delta(const ej_handle* h, uint64_t nR, int planner) {
  if (h->opt_bucket_delta_set) return h->opt_bucket_delta;
  const ej_tune_entry* e = tuning_for(h, nR);
  return e ? e->bucket_delta : planner;
}

int ej_tuned_partition_bits(const ej_handle* h, uint64_t nR) {
  if (h->opt_partition_bits >= 0) return h->opt_partition_bits;
  const ej_tune_entry* e = tuning_for(h, nR);
  return e ? e->partition_bits : -1;
}

int ej_tuned_build(const ej_handle* h, uint64_t nR) {
  if (h->opt_build) return h->opt_build;
  const ej_tune_entry* e = tuning_for(h, nR);
  return e ? e->build : EJ_BUILD_PLANNER;
}

int ej_tuned_table_format(const ej_handle* h, uint64_t nR) {
  if (h->opt_table) return h->opt_table;
  const ej_tune_entry* e = tuning_for(h, nR);
  return e ? e->table : EJ_TABLE_FORMAT_PLANNER;
}

int ej_tuned_probe_warps(const ej_handle* h, uint64_t nR) {
  if (h->opt_probe_warps) return h->opt_probe_warps;
  const ej_tune_entry* e = tuning_for(h, nR);
  return e && e->probe_warps ? e->probe_warps : 8;
}

extern "C" ej_status ej_last_phase_ms(ej_handle* h, float ms[EJ_PHASES]) {
  if (!h || !ms) return EJ_ERR_INVALID;
  for (int i = 0; i < EJ_PHASES; i++) ms[i] = 0.f;
  if (h->last_set < 0) return EJ_OK;
  return set_phases(h, h->last_set, ms);
}

extern "C" ej_status ej_phase_totals(ej_handle* h, double ms[EJ_PHASES], uint32_t* joins) {
  if (!h || !ms) return EJ_ERR_INVALID;
  for (int i = 0; i < EJ_PHASES; i++) ms[i] = 0.0;
  const uint32_t n = h->ring_pending;
  for (uint32_t j = 0; j < n; j++) {
    const int set = (int)((h->ring_head + EJ_PHASE_RING - 1 - (h->cur_set >= 0 ? 1 : 0) - j) % EJ_PHASE_RING);
    float f[EJ_PHASES];
    EJ_TRY(set_phases(h, set, f));
    for (int i = 0; i < EJ_PHASES; i++) ms[i] += f[i];
  }
  h->ring_pending = 0;
  if (joins) *joins = n;
  return EJ_OK;
}

ej_status ej_arena_reserve(ej_handle* h, size_t bytes) {
  h->prep_valid = false;  // every call that lays out the arena overwrites a kept count
  if (bytes <= h->arena_cap) return EJ_OK;
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->arena) EJ_CUDA(h, cudaFree(h->arena));
  h->arena = nullptr;
  h->arena_cap = 0;
  const size_t want = bytes + (bytes >> 4) + ((size_t)1 << 20);
  if (ej_dev_alloc(&h->arena, want) != cudaSuccess) {
    cudaGetLastError();
    h->arena = nullptr;
    return ej_fail(h, EJ_ERR_NOMEM, "device scratch of %zu bytes could not be allocated", want);
  }
  h->arena_cap = want;
  if (want > h->arena_peak) h->arena_peak = want;
  return EJ_OK;
}

ej_status ej_begin(ej_handle* h) {
  if (!h) return EJ_ERR_INVALID;
  h->last_error.clear();
  EJ_CUDA(h, cudaSetDevice(h->device));
  return EJ_OK;
}

// Synchronise, fetch the device count word and status, clear the status.
ej_status ej_finish(ej_handle* h, uint64_t* count) {
  EJ_CUDA(h, cudaMemcpyAsync(h->h_words, h->d_words, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  EJ_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(ej_dev_status), cudaMemcpyDeviceToHost, h->stream));
  EJ_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(ej_dev_status), h->stream));
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (count) *count = h->h_words[0];
  const unsigned int code = h->h_status->code;
  if (code != 0 && code != EJ_ERR_CAPACITY)
    return ej_fail(h, (ej_status)code, "device reported %s (site %u)", ej_status_name((ej_status)code),
                   h->h_status->info);
  return EJ_OK;
}

extern "C" ej_status ej_sync_status(ej_handle* h) {
  EJ_TRY(ej_begin(h));
  EJ_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(ej_dev_status), cudaMemcpyDeviceToHost, h->stream));
  EJ_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(ej_dev_status), h->stream));
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  return (ej_status)h->h_status->code;
}

// ---- argument checks --------------------------------------------------------

static bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

ej_status ej_check_rel(ej_handle* h, const char* name, const ej_tuple* p, uint64_t n) {
  if (n && !p) return ej_fail(h, EJ_ERR_INVALID, "%s is NULL with %llu rows", name, (unsigned long long)n);
  if (p && !aligned(p, 8)) return ej_fail(h, EJ_ERR_INVALID, "%s must be 8-byte aligned", name);
  if (n >= 0xFFFFFFFFull)
    return ej_fail(h, EJ_ERR_TOO_LARGE, "%s has %llu rows; the limit is 2^32-2", name, (unsigned long long)n);
  return EJ_OK;
}

ej_status ej_check_out(ej_handle* h, const void* out, uint64_t cap, const uint64_t* out_count) {
  if (!out_count) return ej_fail(h, EJ_ERR_INVALID, "out_count is NULL");
  if (cap && !out) return ej_fail(h, EJ_ERR_INVALID, "out is NULL with capacity %llu", (unsigned long long)cap);
  if (out && !aligned(out, 16)) return ej_fail(h, EJ_ERR_INVALID, "out must be 16-byte aligned");
  return EJ_OK;
}

ej_status ej_capacity_result(ej_handle* h, uint64_t count, uint64_t cap) {
  if (count > cap)
    return ej_fail(h, EJ_ERR_CAPACITY, "%llu results exceed out_cap %llu", (unsigned long long)count,
                   (unsigned long long)cap);
  return EJ_OK;
}

// ---- hash joins ---------------------------------------------------------------

static ej_status hash_join_sync(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                                ej_result* out, uint64_t out_cap, uint64_t* out_count, int mode) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(ej_check_rel(h, "R", R, nR));
  EJ_TRY(ej_check_rel(h, "S", S, nS));
  if (mode != 2) EJ_TRY(ej_check_out(h, out, out_cap, out_count));
  else if (!out_count) return ej_fail(h, EJ_ERR_INVALID, "out_count is NULL");
  EJ_TRY(ej_hash_join_run(h, R, nR, S, nS, out, out_cap, h->d_words, mode));
  uint64_t count = 0;
  const ej_status fs = ej_finish(h, &count);
  if (fs != EJ_OK) {
    h->prep_valid = false;
    return fs;
  }
  *out_count = count;
  if (mode == 2 && h->prep_valid) {
    h->prep->count_known = true;
    h->prep->count = count;
  }
  return mode == 2 ? EJ_OK : ej_capacity_result(h, count, out_cap);
}

extern "C" ej_status ej_hash_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                                  ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return hash_join_sync(h, R, nR, S, nS, out, out_cap, out_count, 0);
}

extern "C" ej_status ej_hash_join_count(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                        uint64_t nS, uint64_t* out_count) {
  return hash_join_sync(h, R, nR, S, nS, nullptr, 0, out_count, 2);
}

extern "C" ej_status ej_single_hash_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                         uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  return hash_join_sync(h, R, nR, S, nS, out, out_cap, out_count, 1);
}

extern "C" ej_status ej_hash_join_async(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                        uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* d_count) {
  EJ_TRY(ej_begin(h));
  EJ_TRY(ej_check_rel(h, "R", R, nR));
  EJ_TRY(ej_check_rel(h, "S", S, nS));
  if (!d_count) return ej_fail(h, EJ_ERR_INVALID, "d_count is NULL");
  if (out_cap && !out) return ej_fail(h, EJ_ERR_INVALID, "out is NULL");
  if (out && !aligned(out, 16)) return ej_fail(h, EJ_ERR_INVALID, "out must be 16-byte aligned");
  return ej_hash_join_run(h, R, nR, S, nS, out, out_cap, reinterpret_cast<unsigned long long*>(d_count), 0);
}

// ---- generic dispatcher -------------------------------------------------------

extern "C" ej_status ej_join(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  switch (algo) {
    case EJ_ALGO_HASH: return ej_hash_join(h, R, nR, S, nS, out, out_cap, out_count);
    case EJ_ALGO_SINGLE_HASH: return ej_single_hash_join(h, R, nR, S, nS, out, out_cap, out_count);
    case EJ_ALGO_BNL: return ej_bnl_join(h, R, nR, S, nS, out, out_cap, out_count);
    case EJ_ALGO_HASH_INDEX: return ej_hash_index_join(h, R, nR, S, nS, out, out_cap, out_count);
    case EJ_ALGO_SORT_INDEX: return ej_sort_index_join(h, R, nR, S, nS, out, out_cap, out_count);
    case EJ_ALGO_LEFT_OUTER: return ej_left_outer_join(h, R, nR, S, nS, out, out_cap, out_count);
  }
  return ej_fail(h, EJ_ERR_INVALID, "unknown algorithm %d", (int)algo);
}

// ---- host-buffer path ------------------------------------------------------------

// A device address for a host buffer the GPU can store to directly: pinned
// (page-locked, mapped) host memory.  nullptr for pageable memory, which is
// staged through device memory instead.
static void* mapped_view(void* host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

extern "C" ej_status ej_join_host(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                                  uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count) {
  EJ_TRY(ej_begin(h));
  if ((nR && !R) || (nS && !S) || (out_cap && !out) || !out_count) return ej_fail(h, EJ_ERR_INVALID, "null buffer");
  // pinned output: the write pass stores rows straight into host memory over
  // the CPU-GPU link, so no device copy of the output and no download pass
  ej_result* direct = out_cap ? static_cast<ej_result*>(mapped_view(out)) : nullptr;
  if (direct && !aligned(direct, 16)) direct = nullptr;
  ej_plan_bytes p;
  const size_t r_off = p.add(nR * sizeof(ej_tuple));
  const size_t s_off = p.add(nS * sizeof(ej_tuple));
  const size_t o_off = p.add(direct ? 0 : out_cap * sizeof(ej_result));
  if (p.bytes > h->stage_cap) {
    EJ_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->stage) EJ_CUDA(h, cudaFree(h->stage));
    h->stage = nullptr;
    h->stage_cap = 0;
    if (ej_dev_alloc(&h->stage, p.bytes) != cudaSuccess) {
      cudaGetLastError();
      return ej_fail(h, EJ_ERR_NOMEM, "host-path staging of %zu bytes could not be allocated", p.bytes);
    }
    h->stage_cap = p.bytes;
  }
  char* base = static_cast<char*>(h->stage);
  ej_tuple* dR = reinterpret_cast<ej_tuple*>(base + r_off);
  ej_tuple* dS = reinterpret_cast<ej_tuple*>(base + s_off);
  ej_result* dO = direct ? direct : reinterpret_cast<ej_result*>(base + o_off);
  if (nR) EJ_CUDA(h, cudaMemcpyAsync(dR, R, nR * sizeof(ej_tuple), cudaMemcpyHostToDevice, h->stream));
  if (nS) EJ_CUDA(h, cudaMemcpyAsync(dS, S, nS * sizeof(ej_tuple), cudaMemcpyHostToDevice, h->stream));
  uint64_t count = 0;
  ej_status st = ej_join(h, algo, dR, nR, dS, nS, out_cap ? dO : nullptr, out_cap, &count);
  *out_count = count;
  if (st != EJ_OK && st != EJ_ERR_CAPACITY) return st;
  const uint64_t rows = count < out_cap ? count : out_cap;
  if (rows && !direct) {
    EJ_CUDA(h, cudaMemcpyAsync(out, dO, rows * sizeof(ej_result), cudaMemcpyDeviceToHost, h->stream));
    EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return st;
}

// ---- scan ------------------------------------------------------------------------

extern "C" ej_status ej_exclusive_scan_u32(ej_handle* h, const uint32_t* in, uint64_t n, uint64_t* out) {
  EJ_TRY(ej_begin(h));
  if ((n && !in) || !out) return ej_fail(h, EJ_ERR_INVALID, "null buffer");
  ej_plan_bytes p;
  const size_t off = p.add(ej_scan_scratch_bytes(n));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  EJ_TRY(ej_scan_u32_u64(h, in, n, reinterpret_cast<unsigned long long*>(out), ej_arena_at(h, off)));
  return ej_finish(h, nullptr);
}

// ---- generators --------------------------------------------------------------------

namespace {

__global__ void gen_kernel(ej_gen_spec spec, ej_tuple* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < spec.n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t val = ej_gen_val(&spec, i);
    reinterpret_cast<int2*>(out)[i] = make_int2((int32_t)((uint32_t)spec.key_base + (uint32_t)i), val);
  }
}

__global__ void checksum_kernel(const int32_t* __restrict__ w, uint64_t nrows, uint32_t wpr,
                                unsigned long long* __restrict__ acc) {
  __shared__ unsigned long long warp_tmp[256 / 32 + 1];
  unsigned long long sum = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrows;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t hsh = 0x243F6A8885A308D3ull;
    for (uint32_t k = 0; k < wpr; k++) hsh = ej_splitmix64(hsh ^ (uint64_t)(uint32_t)w[i * wpr + k]);
    sum += hsh;
  }
  unsigned long long total;
  ej_block_exclusive_sum<256, unsigned long long>(sum, warp_tmp, &total);
  if (threadIdx.x == 0) atomicAdd(acc, total);
}

// the checksums of many joins' outputs: block (x, y) sums the rows of join x
// at positions y * 256 + t, y * 256 + t + gridDim.y * 256, ...
__global__ void __launch_bounds__(256) checksum_outputs_kernel(const ej_join_desc* __restrict__ d,
                                                               const unsigned long long* __restrict__ counts,
                                                               unsigned long long* __restrict__ sums) {
  __shared__ unsigned long long warp_tmp[256 / 32 + 1];
  const ej_join_desc j = d[blockIdx.x];
  const uint64_t rows = min((uint64_t)counts[blockIdx.x], j.out_cap);
  const int4* out = reinterpret_cast<const int4*>(j.out);
  unsigned long long sum = 0;
  for (uint64_t i = (uint64_t)blockIdx.y * 256 + threadIdx.x; i < rows; i += (uint64_t)gridDim.y * 256) {
    const int4 r = out[i];
    uint64_t hsh = 0x243F6A8885A308D3ull;
    hsh = ej_splitmix64(hsh ^ (uint64_t)(uint32_t)r.x);
    hsh = ej_splitmix64(hsh ^ (uint64_t)(uint32_t)r.y);
    hsh = ej_splitmix64(hsh ^ (uint64_t)(uint32_t)r.z);
    sum += ej_splitmix64(hsh ^ (uint64_t)(uint32_t)r.w);
  }
  unsigned long long total;
  ej_block_exclusive_sum<256, unsigned long long>(sum, warp_tmp, &total);
  if (threadIdx.x == 0 && total) atomicAdd(sums + blockIdx.x, total);
}

}  // namespace

ej_status ej_checksum_outputs_async(ej_handle* h, const ej_join_desc* d_desc, const unsigned long long* d_counts,
                                    uint32_t n, unsigned long long* d_sums) {
  if (!n) return EJ_OK;
  EJ_CUDA(h, cudaMemsetAsync(d_sums, 0, n * sizeof(unsigned long long), h->stream));
  checksum_outputs_kernel<<<dim3(n, 32), 256, 0, h->stream>>>(d_desc, d_counts, d_sums);
  return ej_check_launch(h, "checksum_outputs_kernel");
}

// Zipf CDF over ranks 1..n with exponent s, built on the host in double
// precision (the oracle builds its table with the same loop).
static void zipf_cdf_host(double s, uint32_t n, double* cdf) {
  double total = 0.0;
  for (uint32_t k = 0; k < n; k++) {
    total += std::pow((double)(k + 1u), -s);
    cdf[k] = total;
  }
  for (uint32_t k = 0; k < n; k++) cdf[k] = cdf[k] / total;
  if (n) cdf[n - 1] = 1.0;
}

extern "C" ej_status ej_generate(ej_handle* h, const ej_gen_spec* spec, ej_tuple* out) {
  EJ_TRY(ej_begin(h));
  if (!spec) return ej_fail(h, EJ_ERR_INVALID, "spec is NULL");
  EJ_TRY(ej_check_rel(h, "out", out, spec->n));
  if (spec->kind > EJ_GEN_ZIPF || spec->domain == 0)
    return ej_fail(h, EJ_ERR_INVALID, "bad generator spec (kind %u, domain %u)", spec->kind, spec->domain);
  ej_gen_spec sp = *spec;
  if (sp.kind == EJ_GEN_PERM) {
    const uint32_t dup = sp.dup ? sp.dup : 1u;
    if ((sp.n + dup - 1) / dup > sp.domain)
      return ej_fail(h, EJ_ERR_INVALID, "PERM spec needs n/dup <= domain");
  }
  if (sp.kind == EJ_GEN_ZIPF && sp.zipf_s != 0.0 && !sp.cdf) {
    if (h->zipf.s != sp.zipf_s || h->zipf.domain != sp.domain || !h->zipf.d_cdf) {
      std::vector<double> cdf(sp.domain);
      zipf_cdf_host(sp.zipf_s, sp.domain, cdf.data());
      EJ_CUDA(h, cudaStreamSynchronize(h->stream));
      cudaFree(h->zipf.d_cdf);
      h->zipf.d_cdf = nullptr;
      EJ_CUDA(h, ej_dev_alloc(&h->zipf.d_cdf, sizeof(double) * sp.domain));
      EJ_CUDA(h, cudaMemcpy(h->zipf.d_cdf, cdf.data(), sizeof(double) * sp.domain, cudaMemcpyHostToDevice));
      h->zipf.s = sp.zipf_s;
      h->zipf.domain = sp.domain;
    }
    sp.cdf = h->zipf.d_cdf;
  }
  if (sp.n) {
    const unsigned blocks = (unsigned)std::min<uint64_t>((sp.n + 255) / 256, (uint64_t)h->num_sms * 32);
    gen_kernel<<<blocks, 256, 0, h->stream>>>(sp, out);
    EJ_TRY(ej_check_launch(h, "gen_kernel"));
  }
  return ej_finish(h, nullptr);
}

extern "C" ej_status ej_checksum(ej_handle* h, const void* rows, uint64_t nrows, uint32_t words_per_row,
                                 uint64_t* out_sum) {
  EJ_TRY(ej_begin(h));
  if ((nrows && !rows) || !out_sum || words_per_row == 0) return ej_fail(h, EJ_ERR_INVALID, "bad checksum args");
  EJ_CUDA(h, cudaMemsetAsync(h->d_words, 0, sizeof(unsigned long long), h->stream));
  if (nrows) {
    const unsigned blocks = (unsigned)std::min<uint64_t>((nrows + 255) / 256, (uint64_t)h->num_sms * 16);
    checksum_kernel<<<blocks, 256, 0, h->stream>>>(static_cast<const int32_t*>(rows), nrows, words_per_row,
                                                   h->d_words);
    EJ_TRY(ej_check_launch(h, "checksum_kernel"));
  }
  uint64_t v = 0;
  EJ_TRY(ej_finish(h, &v));
  *out_sum = v;
  return EJ_OK;
}
