// ej_device.cuh - device helpers: hashing, bounded waits, warp/block scans.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ej_internal.h"

#define EJ_FULL_MASK 0xFFFFFFFFu

// Bounded device waits give up after a limit in nanoseconds of %globaltimer
// (the handle's, EJ_DEFAULT_WAIT_LIMIT_NS unless set) and report
// EJ_ERR_TIMEOUT through the status word instead of hanging.

// 32-bit finaliser of MurmurHash3 (Appleby, public domain): a bijection on
// uint32, so distinct keys keep distinct hashes and buckets/partitions are
// taken from its top bits.
__device__ __forceinline__ uint32_t ej_hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ unsigned long long ej_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ej_lanemask_lt() {
  unsigned int m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned long long ej_ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void ej_st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Record the first device error (later errors keep the first one).
__device__ __forceinline__ void ej_set_status(ej_dev_status* st, unsigned int code, unsigned int info) {
  if (st && atomicCAS(&st->code, 0u, code) == 0u) st->info = info;
}

// Lanes of the warp whose BITS-bit digit equals this lane's, restricted to
// `valid` lanes: one ballot per digit bit, each narrowing the candidate set to
// the lanes that agree on that bit.  Same result as __match_any_sync on the
// digit, at a fraction of its issue cost for digits of up to 8 bits.
template <int BITS>
__device__ __forceinline__ unsigned int ej_match_digit(uint32_t d, unsigned int valid) {
  unsigned int peers = valid;
#pragma unroll
  for (int b = 0; b < BITS; b++) {
    const bool bit = (d >> b) & 1u;
    const unsigned int m = __ballot_sync(EJ_FULL_MASK, bit);
    peers &= bit ? m : ~m;
  }
  return peers;
}

template <typename T>
__device__ __forceinline__ T ej_warp_inclusive_sum(T v) {
  const unsigned int lane = threadIdx.x & 31u;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = __shfl_up_sync(EJ_FULL_MASK, v, d);
    if (lane >= (unsigned)d) v += o;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T ej_warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(EJ_FULL_MASK, v, d);
  return v;
}

// Block-wide exclusive sum for THREADS threads (multiple of 32, <= 1024).
// `warp_tmp` is shared scratch of THREADS/32 + 1 elements.  Returns the
// thread's exclusive prefix; *total receives the block total (all threads).
template <int THREADS, typename T>
__device__ __forceinline__ T ej_block_exclusive_sum(T v, T* warp_tmp, T* total) {
  constexpr int WARPS = THREADS / 32;
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  T incl = ej_warp_inclusive_sum(v);
  if (lane == 31u) warp_tmp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (unsigned)WARPS ? warp_tmp[lane] : T(0);
    T wi = ej_warp_inclusive_sum(w);
    if (lane < (unsigned)WARPS) warp_tmp[lane] = wi - w;
    if (lane == (unsigned)WARPS - 1) warp_tmp[WARPS] = wi;
  }
  __syncthreads();
  T r = warp_tmp[warp] + incl - v;
  *total = warp_tmp[WARPS];
  __syncthreads();
  return r;
}

// Decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix Scan
// with Decoupled Look-back", NVIDIA TR 2016).  Status words pack a 2-bit flag
// (0 = not ready, 1 = tile aggregate, 2 = inclusive prefix) over a 62-bit value.
// Tiles take ids in launch order from an atomic counter, so a tile only ever
// waits for tiles that have already started; the wait is still bounded.
#define EJ_LB_AGG 1ull
#define EJ_LB_PREFIX 2ull
#define EJ_LB_VALUE_MASK ((1ull << 62) - 1ull)

// Both halves are called by one full warp; the exclusive prefix is returned
// in every lane.  The two halves of a look-back step, so that a tile can do
// other work between them: publish the tile's aggregate (tile 0: its
// inclusive prefix)...
__device__ __forceinline__ void ej_lookback_publish(unsigned long long* status, uint64_t tile,
                                                    unsigned long long aggregate) {
  if ((threadIdx.x & 31u) == 0)
    ej_st_relaxed(&status[tile], ((tile == 0 ? EJ_LB_PREFIX : EJ_LB_AGG) << 62) | (aggregate & EJ_LB_VALUE_MASK));
}

// ...then walk back over the predecessors (32 per step, one per lane) until
// one with an inclusive prefix, publish this tile's inclusive prefix and
// return its exclusive one.  A wait longer than limit_ns takes the missing
// predecessors as zero and records EJ_ERR_TIMEOUT at `where`; prefixes then
// come out too small, never too large, so positions derived from them stay
// inside their buffers.  The clock is read every 64 polls, every poll when
// the limit is under 100 us (limit 0: give up at the first poll that finds a
// predecessor not ready).
__device__ __forceinline__ unsigned long long ej_lookback_resolve(unsigned long long* status, uint64_t tile,
                                                                  unsigned long long aggregate,
                                                                  ej_dev_status* st, unsigned int where,
                                                                  unsigned long long limit_ns) {
  const unsigned int lane = threadIdx.x & 31u;
  if (tile == 0) return 0ull;
  unsigned long long exclusive = 0;
  int64_t k = (int64_t)tile - 1;
  const unsigned long long t0 = ej_globaltimer();
  const unsigned int period = limit_ns < 100000ull ? 0u : 63u;
  bool gave_up = false;
  for (;;) {
    const int64_t idx = k - (int64_t)lane;
    unsigned long long w = idx >= 0 ? ej_ld_relaxed(&status[idx]) : (EJ_LB_PREFIX << 62);
    unsigned int spins = 0;
    while (__any_sync(EJ_FULL_MASK, (w >> 62) == 0ull)) {
      if ((w >> 62) == 0ull) {
        __nanosleep(spins < 8 ? 32u : 256u);
        w = ej_ld_relaxed(&status[idx]);
      }
      spins++;
      bool late = false;
      if ((spins & period) == 0u) late = (ej_globaltimer() - t0) >= limit_ns;
      if (__shfl_sync(EJ_FULL_MASK, late ? 1 : 0, 0)) {
        gave_up = true;
        if ((w >> 62) == 0ull) w = (EJ_LB_PREFIX << 62);
      }
    }
    const unsigned int prefix_lanes = __ballot_sync(EJ_FULL_MASK, (w >> 62) == EJ_LB_PREFIX);
    unsigned long long v = w & EJ_LB_VALUE_MASK;
    if (prefix_lanes) {
      const unsigned int first = __ffs(prefix_lanes) - 1u;
      exclusive += ej_warp_sum(lane <= first ? v : 0ull);
      break;
    }
    exclusive += ej_warp_sum(v);
    k -= 32;
  }
  if (lane == 0) {
    ej_st_relaxed(&status[tile], (EJ_LB_PREFIX << 62) | ((exclusive + aggregate) & EJ_LB_VALUE_MASK));
    if (gave_up) ej_set_status(st, EJ_ERR_TIMEOUT, where);
  }
  return exclusive;
}

// both halves at once
__device__ __forceinline__ unsigned long long ej_lookback_warp(unsigned long long* status, uint64_t tile,
                                                             unsigned long long aggregate,
                                                             ej_dev_status* st, unsigned int where,
                                                             unsigned long long limit_ns) {
  ej_lookback_publish(status, tile, aggregate);
  return ej_lookback_resolve(status, tile, aggregate, st, where, limit_ns);
}
