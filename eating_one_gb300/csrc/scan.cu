// scan.cu - single-pass exclusive prefix sum with decoupled look-back.
//
// Replaces the reference's presum()/scanExclusive* (NVIDIA-sample 3-level
// scan, joins/hashJoin_gpu/main_street/scan_main.cpp:38-111, scan.cu:88-227),
// which pads its input, launches 3-5 kernels, allocates and frees per call and
// replaces its input buffer.  Here: one launch, inputs untouched, n+1 outputs
// (the last one is the total, so no separate getValue readback kernel,
// scan_main.cpp:160-180), 64-bit outputs where totals can exceed 2^32.
#include <mutex>

#include "ej_device.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename In, typename Out>
__global__ void __launch_bounds__(SCAN_THREADS)
scan_kernel(const In* __restrict__ in, uint64_t n, Out* __restrict__ out, unsigned long long* status,
            unsigned int* tile_ctr, uint64_t ntiles, ej_dev_status* st, unsigned long long wait_ns) {
  __shared__ Out sbuf[SCAN_TILE + SCAN_TILE / 32];
  __shared__ Out warp_tmp[SCAN_THREADS / 32 + 1];
  __shared__ unsigned int s_tile;
  __shared__ Out s_prefix;

  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint64_t base = tile * SCAN_TILE;

  // striped (coalesced) load, transposed through shared memory to a blocked layout
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    const int s = i * SCAN_THREADS + threadIdx.x;
    const uint64_t idx = base + (uint64_t)s;
    sbuf[s + (s >> 5)] = idx < n ? (Out)in[idx] : (Out)0;
  }
  __syncthreads();
  Out v[SCAN_ITEMS];
  Out sum = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; j++) {
    const int s = threadIdx.x * SCAN_ITEMS + j;
    v[j] = sbuf[s + (s >> 5)];
    sum += v[j];
  }
  Out aggregate;
  const Out thread_excl = ej_block_exclusive_sum<SCAN_THREADS, Out>(sum, warp_tmp, &aggregate);

  if (threadIdx.x < 32) {
    const unsigned long long ex =
        ej_lookback_warp(status, tile, (unsigned long long)aggregate, st, /*where=*/1u, wait_ns);
    if (threadIdx.x == 0) s_prefix = (Out)ex;
  }
  __syncthreads();

  Out run = s_prefix + thread_excl;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; j++) {
    const int s = threadIdx.x * SCAN_ITEMS + j;
    sbuf[s + (s >> 5)] = run;
    run += v[j];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    const int s = i * SCAN_THREADS + threadIdx.x;
    const uint64_t idx = base + (uint64_t)s;
    if (idx < n) out[idx] = sbuf[s + (s >> 5)];
  }
  if (tile == ntiles - 1 && threadIdx.x == 0) out[n] = s_prefix + aggregate;
}

template <typename In, typename Out>
ej_status launch_scan(ej_handle* h, const In* in, uint64_t n, Out* out, void* scratch) {
  if (n == 0) {
    EJ_CUDA(h, cudaMemsetAsync(out, 0, sizeof(Out), h->stream));
    return EJ_OK;
  }
  const uint64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles > 0xFFFFFFFFull) return ej_fail(h, EJ_ERR_TOO_LARGE, "scan: %llu elements", (unsigned long long)n);
  unsigned long long* status = static_cast<unsigned long long*>(scratch);
  unsigned int* ctr = reinterpret_cast<unsigned int*>(status + ntiles);
  EJ_CUDA(h, cudaMemsetAsync(scratch, 0, ntiles * sizeof(unsigned long long) + 16, h->stream));
  scan_kernel<In, Out><<<(unsigned)ntiles, SCAN_THREADS, 0, h->stream>>>(in, n, out, status, ctr, ntiles,
                                                                         h->d_status, h->wait_limit_ns);
  return ej_check_launch(h, "scan_kernel");
}

}  // namespace

size_t ej_scan_scratch_bytes(uint64_t n) {
  const uint64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  return (size_t)(ntiles * sizeof(unsigned long long) + 16);
}

ej_status ej_scan_u32_u32(ej_handle* h, const uint32_t* in, uint64_t n, uint32_t* out, void* scratch) {
  return launch_scan<uint32_t, uint32_t>(h, in, n, out, scratch);
}

ej_status ej_scan_u32_u64(ej_handle* h, const uint32_t* in, uint64_t n, unsigned long long* out,
                          void* scratch) {
  return launch_scan<uint32_t, unsigned long long>(h, in, n, out, scratch);
}

ej_status ej_scan_u64_u64(ej_handle* h, const unsigned long long* in, uint64_t n,
                          unsigned long long* out, void* scratch) {
  return launch_scan<unsigned long long, unsigned long long>(h, in, n, out, scratch);
}

// ---- scan without allocation ------------------------------------------------
// For callers that cannot allocate device memory (their framework owns the
// GPU's memory, they must not trigger the device-wide synchronisation of
// cudaMalloc/cudaFree, or they cannot keep a handle).  The look-back scratch
// is this file-scope array instead of handle memory; every device that loads
// the library holds it until the process exits.

namespace {

constexpr uint64_t NOALLOC_TILES = (EJ_NOALLOC_SCAN_MAX_N + SCAN_TILE - 1) / SCAN_TILE;  // 65536
constexpr int NOALLOC_MAX_DEVICES = 64;

// look-back status words of every tile, then one word holding the tile counter
static __device__ __align__(256) unsigned long long g_noalloc_scan_scratch[NOALLOC_TILES + 1];
// device status word of the no-allocation scan (bounded-wait timeouts)
static __device__ __align__(256) ej_dev_status g_noalloc_scan_status;

struct NoallocDevice {
  bool ready = false;
  unsigned long long* scratch = nullptr;  // device address of g_noalloc_scan_scratch
  ej_dev_status* status = nullptr;        // device address of g_noalloc_scan_status
};
NoallocDevice g_noalloc_devices[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mutex;

}  // namespace

extern "C" ej_status ej_exclusive_scan_u32_noalloc(const uint32_t* in, uint64_t n, uint64_t* out,
                                                   ej_stream stream) {
  if ((n && !in) || !out) return EJ_ERR_INVALID;
  if (n > EJ_NOALLOC_SCAN_MAX_N) return EJ_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return EJ_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return EJ_ERR_INVALID;
  NoallocDevice& d = g_noalloc_devices[dev];
  {
    // set-up once per device, with that device current: the host-side names of
    // the static arrays are not device addresses, so look the addresses up
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!d.ready) {
      void* scratch = nullptr;
      void* status = nullptr;
      if (cudaGetSymbolAddress(&scratch, g_noalloc_scan_scratch) != cudaSuccess ||
          cudaGetSymbolAddress(&status, g_noalloc_scan_status) != cudaSuccess) {
        cudaGetLastError();
        return EJ_ERR_CUDA;
      }
      d.scratch = static_cast<unsigned long long*>(scratch);
      d.status = static_cast<ej_dev_status*>(status);
      d.ready = true;
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
  if (n == 0) {
    if (cudaMemsetAsync(o, 0, sizeof(unsigned long long), s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cudaGetLastError();
      return EJ_ERR_CUDA;
    }
    return EJ_OK;
  }
  const uint64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  // the array keeps the previous call's words: clear the status words, the
  // tile counter and the status word before every launch
  if (cudaMemsetAsync(d.scratch, 0, (ntiles + 1) * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(d.status, 0, sizeof(ej_dev_status), s) != cudaSuccess) {
    cudaGetLastError();
    return EJ_ERR_CUDA;
  }
  unsigned int* ctr = reinterpret_cast<unsigned int*>(d.scratch + ntiles);
  scan_kernel<uint32_t, unsigned long long><<<(unsigned)ntiles, SCAN_THREADS, 0, s>>>(
      in, n, o, d.scratch, ctr, ntiles, d.status, EJ_DEFAULT_WAIT_LIMIT_NS);
  if (cudaGetLastError() != cudaSuccess) return EJ_ERR_CUDA;
  ej_dev_status host_status;
  if (cudaMemcpyAsync(&host_status, d.status, sizeof(host_status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return EJ_ERR_CUDA;
  }
  return host_status.code ? (ej_status)host_status.code : EJ_OK;
}
