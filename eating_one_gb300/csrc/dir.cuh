// dir.cuh - the key directory of a hash table (device code): the build's
// per-tile steps, shared by single tables (hash_join.cu) and the tables of a
// batch (batch.cu).
//
// The distinct keys of the hash-sorted table, in hash order, each an entry
// {hash, run start} placed by linear probing from its home slot, the even
// slot (hash >> (32 - bits)) & ~1 (2^bits >= 4 x keys where the reserved
// slots allow, else as many as they hold): key k goes to
//   pos_k = max(home_k, pos_{k-1} + 1) = k + max_{j <= k} (home_j - j),
// so the entries stay in hash order.  A probe loads the aligned 16-byte pair
// of slots at its home, so that it needs a second load only when both hold
// smaller hashes (about 4% of probes at a quarter of the slots filled).  Tables under 2^27 rows pack an entry
// as {hash, start << 5 | run length} (31: 31 rows or more, the run then ends
// at the next slot's start), so that one 8-byte load answers most probes;
// larger tables keep {hash, start}.  Every slot holds the first key at or
// after it: the slots between pos_{k-1} and pos_k hold copies of key k, the
// slots past the last entry a sentinel {0xFFFFFFFF, nR}.  A probe walks
// forward from its home slot past smaller hashes; it has found its key when
// the hash matches and the start is below nR, and the run ends at the first
// later slot whose start differs (the next key's start).  The number of keys,
// and so bits, is known only on the device: it lives in a header.  Build, per
// table: per 4096-row tile, count the rows that begin a key; scan; per tile,
// the largest home_k - k; a prefix maximum over the tiles; per tile, every
// key's slots (pos_{k-1}, pos_k]; then the slots before the first entry and
// after the last.
#pragma once

#include <climits>

#include "ej_device.cuh"

constexpr int DIR_ROWS = 16;              // consecutive rows per thread
constexpr int DIR_THREADS = 256;
constexpr int DIR_TILE = DIR_THREADS * DIR_ROWS;  // rows per tile (one block)

struct DirHeader {
  uint32_t bits;
  uint32_t hash0;  // hash of the first key
  unsigned long long nkeys;
  unsigned long long pos_first, pos_last;  // slots of the first and last entries
  uint32_t lead;  // packed entries: the first key's {start << 5 | run length}
  uint32_t pad;
};
constexpr size_t DIR_HEADER_BYTES = 256;

// directory slots reserved for nR rows: 2^bits <= next power of two of 2 nR,
// plus one slot per key for the entries past the last home slot, plus two
// sentinels (the last written slot is at most 2^bits + keys)
inline uint64_t ej_dir_capacity(uint64_t nR) {
  uint64_t p = 2;
  while (p < 2 * nR) p <<= 1;
  return p + nR + 2;
}

// DIR_ROWS consecutive rows of a thread: vals and which of them begin a key
struct DirRows {
  int32_t v[DIR_ROWS];
  uint32_t f;  // bit e: row i0 + e begins a key
};

__device__ __forceinline__ void dir_rows(const int32_t* __restrict__ rval, uint64_t n, uint64_t i0, DirRows& r) {
  r.f = 0;
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++) r.v[e] = 0;
  if (i0 >= n) return;
  int32_t prev = i0 ? rval[i0 - 1] : 0;
  if (i0 + DIR_ROWS <= n && (reinterpret_cast<uintptr_t>(rval + i0) & 15u) == 0) {
    // a full run of rows at a 16-byte boundary (the columns start aligned
    // and tiles begin at multiples of DIR_ROWS rows): four 16-byte loads
    const int4* c4 = reinterpret_cast<const int4*>(rval + i0);
#pragma unroll
    for (int q = 0; q < DIR_ROWS / 4; q++) {
      const int4 x = c4[q];
      r.v[4 * q] = x.x;
      r.v[4 * q + 1] = x.y;
      r.v[4 * q + 2] = x.z;
      r.v[4 * q + 3] = x.w;
    }
#pragma unroll
    for (int e = 0; e < DIR_ROWS; e++) {
      if (i0 + e == 0 || r.v[e] != prev) r.f |= 1u << e;
      prev = r.v[e];
    }
    return;
  }
  // the table's last rows
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++)
    if (i0 + e < n) r.v[e] = rval[i0 + e];
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++) {
    if (i0 + e < n && (i0 + e == 0 || r.v[e] != prev)) r.f |= 1u << e;
    prev = r.v[e];
  }
}

// bits of a directory of nk keys in a table of n rows: 2^bits >= 4 nk, at most
// the power of two ej_dir_capacity(n) reserves (>= 2 n >= 2 nk)
__device__ __forceinline__ uint32_t dir_bits_for(unsigned long long nk, unsigned long long n) {
  uint32_t bits = 1;
  while (bits < 32 && (1ull << bits) < 4 * nk && (1ull << bits) < 2 * n) bits++;
  return bits;
}

// home slot of a hash: even, so that its pair is one aligned 16-byte load
__device__ __forceinline__ uint32_t dir_home(uint32_t hv, uint32_t shift) { return (hv >> shift) & ~1u; }

// block-wide maximum scan, exclusive (LLONG_MIN for thread 0); *total = the block maximum
__device__ __forceinline__ long long dir_block_exclusive_max(long long v, long long* tmp, long long* total) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (unsigned)o) incl = max(incl, u);
  }
  if (lane == 31u) tmp[warp] = incl;
  __syncthreads();
  long long before = LLONG_MIN;
  for (unsigned w = 0; w < warp; w++) before = max(before, tmp[w]);
  long long all = LLONG_MIN;
  for (unsigned w = 0; w < nw; w++) all = max(all, tmp[w]);
  const long long up = __shfl_up_sync(0xffffffffu, incl, 1);
  const long long ex = max(before, lane ? up : LLONG_MIN);
  __syncthreads();
  *total = all;
  return ex;
}

// the tile at row0 of a table of n rows: rows beginning a key (block total)
__device__ __forceinline__ uint32_t dir_tile_keys(const int32_t* __restrict__ rval, uint64_t n, uint64_t row0) {
  __shared__ uint32_t tmp[DIR_THREADS / 32 + 1];
  DirRows r;
  dir_rows(rval, n, row0 + threadIdx.x * DIR_ROWS, r);
  uint32_t total;
  ej_block_exclusive_sum<DIR_THREADS, uint32_t>((uint32_t)__popc(r.f), tmp, &total);
  return total;
}

// the tile at row0, whose first key has rank k0: the largest home_k - k (block
// maximum; LLONG_MIN when the tile begins no key); hash0 gets the first key's
// hash when row0 == 0
__device__ __forceinline__ long long dir_tile_max(const int32_t* __restrict__ rval, uint64_t n, uint64_t row0,
                                                  uint64_t k0, uint32_t bits, uint32_t* hash0) {
  __shared__ uint32_t tmp[DIR_THREADS / 32 + 1];
  __shared__ long long tmpl[DIR_THREADS / 32];
  DirRows r;
  dir_rows(rval, n, row0 + threadIdx.x * DIR_ROWS, r);
  uint32_t total;
  uint64_t k = k0 + ej_block_exclusive_sum<DIR_THREADS, uint32_t>((uint32_t)__popc(r.f), tmp, &total);
  const uint32_t shift = 32u - bits;
  long long m = LLONG_MIN;
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++)
    if (r.f >> e & 1u) {
      m = max(m, (long long)dir_home(ej_hash32((uint32_t)r.v[e]), shift) - (long long)k);
      k++;
    }
  if (row0 == 0 && threadIdx.x == 0) *hash0 = ej_hash32((uint32_t)r.v[0]);  // row 0 begins the first key
  long long all;
  dir_block_exclusive_max(m, tmpl, &all);
  return all;
}

// slots of a tile's keys staged in shared memory, written out together
constexpr int DIR_STAGE_SLOTS = 5120;  // 40 KB

// the tile at row0 (first key rank k0, largest home_j - j of the keys before
// it: kpre): every key's slots (pos_{k-1}, pos_k], holding {hash_k, start_k}
// or, packed, {hash_k, start_k << 5 | min(run length, 31)}; the first and
// last keys record their slots in the header.  The tile's slots are one
// range, (pos_{k0-1}, pos of its last key]: when it fits DIR_STAGE_SLOTS
// (every tile but the first, whose leading slots dir_edges writes) the
// entries are placed in shared memory and the range leaves in coalesced
// stores, else each thread stores its keys' slots itself.
__device__ __forceinline__ void dir_tile_place(const int32_t* __restrict__ rval, uint64_t n, uint64_t row0,
                                               uint64_t k0, long long kpre, DirHeader* hdr, uint2* __restrict__ dir,
                                               bool packed) {
  __shared__ uint32_t tmp[DIR_THREADS / 32 + 1];
  __shared__ long long tmpl[DIR_THREADS / 32];
  __shared__ uint2 stage[DIR_STAGE_SLOTS];
  const uint64_t i0 = row0 + threadIdx.x * DIR_ROWS;
  DirRows r;
  dir_rows(rval, n, i0, r);
  uint32_t total;
  uint64_t k = k0 + ej_block_exclusive_sum<DIR_THREADS, uint32_t>((uint32_t)__popc(r.f), tmp, &total);
  const unsigned long long nk = hdr->nkeys;
  const uint32_t shift = 32u - hdr->bits;
  long long m = LLONG_MIN;
  uint64_t kk = k;
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++)
    if (r.f >> e & 1u) {
      m = max(m, (long long)dir_home(ej_hash32((uint32_t)r.v[e]), shift) - (long long)kk);
      kk++;
    }
  long long all;
  long long run = max(kpre, dir_block_exclusive_max(m, tmpl, &all));  // max over keys before k
  long long prev = k ? (long long)k - 1 + run : -1;                   // pos_{k-1}
  // the tile's range of slots: from one past pos_{k0-1} to the largest pos
  // of its keys (a thread's last key: its rank plus its running maximum)
  long long last;
  dir_block_exclusive_max(r.f ? (long long)(k + __popc(r.f) - 1) + max(run, m) : LLONG_MIN, tmpl, &last);
  const long long base = (long long)k0 + kpre;  // pos_{k0-1} + 1
  const bool staged = k0 > 0 && total > 0 && last - base < (long long)DIR_STAGE_SLOTS;
  // a key's run ends at the thread's next key, else at the thread's last row
  // plus `tail`: the rows after the thread's that continue its last key
  // (counted up to a run of 31)
  const uint32_t rows = i0 < n ? (uint32_t)min((uint64_t)DIR_ROWS, n - i0) : 0u;
  uint32_t tail = 0;
  if (packed && r.f) {
    int32_t lastv = 0;
    uint32_t lastlen = 0;
#pragma unroll
    for (int e = 0; e < DIR_ROWS; e++)
      if (r.f >> e & 1u) {
        lastv = r.v[e];
        lastlen = rows - e;
      }
    for (uint64_t i = i0 + DIR_ROWS; i < n && lastlen + tail < 31u && rval[i] == lastv; i++) tail++;
  }
#pragma unroll
  for (int e = 0; e < DIR_ROWS; e++) {
    if (!(r.f >> e & 1u)) continue;
    const uint32_t hv = ej_hash32((uint32_t)r.v[e]);
    run = max(run, (long long)dir_home(hv, shift) - (long long)k);
    const long long pos = (long long)k + run;
    const uint32_t rest = r.f >> e >> 1;  // the thread's later keys
    const uint32_t len = rest ? (uint32_t)__ffs(rest) : rows - e + tail;
    const uint32_t y = packed ? (uint32_t)(i0 + e) << 5 | min(len, 31u) : (uint32_t)(i0 + e);
    const uint2 entry = make_uint2(hv, y);
    // key 0's leading slots [0, pos_0) are written by dir_edges
    if (staged)
      for (long long g = prev + 1; g <= pos; g++) stage[g - base] = entry;
    else
      for (long long g = (k ? prev + 1 : pos); g <= pos; g++) dir[g] = entry;
    if (k == 0) {
      hdr->pos_first = (unsigned long long)pos;
      hdr->lead = y;
    }
    if (k + 1 == nk) hdr->pos_last = (unsigned long long)pos;
    prev = pos;
    k++;
  }
  if (staged) {
    __syncthreads();
    const uint32_t w = (uint32_t)(last - base + 1);
    for (uint32_t i = threadIdx.x; i < w; i += DIR_THREADS) dir[base + i] = stage[i];
  }
}

// the slots before the first entry (copies of the first key) and from one
// past the last entry to 2^bits + 1, at least two of them (sentinels
// {0xFFFFFFFF, n}, packed {0xFFFFFFFF, n << 5}; a probe may read the slot
// after the one it stops at); with no keys, slots [0, 2^bits + 1]; threads
// i0, i0 + stride, ... of the caller
__device__ __forceinline__ void dir_edges(const DirHeader* __restrict__ hdr, uint64_t n, uint2* __restrict__ dir,
                                          uint64_t i0, uint64_t stride, bool packed) {
  const unsigned long long home_end = 1ull << hdr->bits;
  const bool any = hdr->nkeys != 0;
  const unsigned long long first = any ? hdr->pos_first : 0ull;
  const unsigned long long tail = any ? hdr->pos_last + 1 : 0ull;
  const unsigned long long tail_end = max(home_end, tail) + 2;
  const uint2 lead = make_uint2(hdr->hash0, packed ? hdr->lead : 0u);
  const uint2 sentinel = make_uint2(0xFFFFFFFFu, packed ? (uint32_t)n << 5 : (uint32_t)n);
  for (uint64_t i = i0; i < first; i += stride) dir[i] = lead;
  for (uint64_t i = tail + i0; i < tail_end; i += stride) dir[i] = sentinel;
}
