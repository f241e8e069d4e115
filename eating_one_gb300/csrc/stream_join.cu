// stream_join.cu - out-of-core joins of host buffers: R in device-sized
// blocks, S streamed through the device in double-buffered chunks.
//
// Replaces the reference drivers' whole-relation upload and download around
// the kernels (joins/hashJoin_gpu/main_street/hj.cc:345-354 cuMemcpyHtoD of
// both relations, :1124 cuMemcpyDtoH of the result) and the block nested
// loop's tiling of the relations into device-sized blocks
// (joins/blockJoin_gpu/main_street/nestLoopJoin.cc:326-519), for relations
// and results of any size.
//
// For each block of at most r_block R rows: upload it (hash join: build its
// table once), then stream S in chunks of at most s_chunk rows:
//   upload stream  : S chunk i+1 ...........................
//   compute stream :      chunk i: [partition] count | write
//   download stream:                   rows of chunk i-1 ....
// Pinned host buffers (cudaHostAlloc / cudaHostRegister) are used in place:
// S chunks are copied straight from S, and the write pass stores rows straight
// into a pinned out over the CPU-GPU link (no device output buffer, no
// download).  Pageable inputs go through two pinned bounce buffers; pageable
// output through two device row buffers and a download.
// Rows are appended in (R block, S chunk) order, so the result multiset is
// the in-core join's; rows beyond out_cap are counted, not written, and the
// call then returns EJ_ERR_CAPACITY with the full count.
#include <string.h>

#include <algorithm>

#include "ej_entry.h"
#include "ej_internal.h"
#include "hash_join.cuh"

enum {
  SR_R_READY,
  SR_BLOCK_DONE,
  SR_S_READY,      // + buffer
  SR_S_FREE = SR_S_READY + 2,
  SR_O_READY = SR_S_FREE + 2,
  SR_O_FREE = SR_O_READY + 2,
  SR_PIN_FREE = SR_O_FREE + 2,
  SR_COUNT = SR_PIN_FREE + 2,
  SR_EVENTS
};

struct ej_stream_res {
  cudaStream_t up = nullptr, down = nullptr;  // host-to-device and device-to-host copies
  cudaEvent_t ev[SR_EVENTS] = {};
  void* dev = nullptr;  // R block, then two S chunk buffers
  size_t dev_cap = 0;
  void* obuf = nullptr;  // two device row buffers (pageable out)
  uint64_t obuf_rows = 0;
  void* pin[2] = {nullptr, nullptr};  // pinned bounce buffers (pageable inputs)
  size_t pin_cap = 0;
};

void ej_stream_release(ej_handle* h) {
  ej_stream_res* r = h->sres;
  if (!r) return;
  if (r->up) cudaStreamSynchronize(r->up);
  if (r->down) cudaStreamSynchronize(r->down);
  for (cudaEvent_t e : r->ev)
    if (e) cudaEventDestroy(e);
  if (r->up) cudaStreamDestroy(r->up);
  if (r->down) cudaStreamDestroy(r->down);
  cudaFree(r->dev);
  cudaFree(r->obuf);
  for (void* p : r->pin) cudaFreeHost(p);
  delete r;
  h->sres = nullptr;
}

namespace {

constexpr uint64_t SJ_DEFAULT_CHUNK = 1ull << 25;  // S rows per chunk (256 MiB)
constexpr size_t SJ_BOUNCE = (size_t)32 << 20;     // bytes per pinned bounce buffer
constexpr uint64_t SJ_MAX_ROWS = 0xFFFFFFFEull;    // rows of one device relation

bool sj_pinned(const void* p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// device address of pinned, mapped host memory; nullptr otherwise
void* sj_mapped(void* p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

ej_status sj_idle(ej_handle* h, ej_stream_res* r) {
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));
  EJ_CUDA(h, cudaStreamSynchronize(r->up));
  EJ_CUDA(h, cudaStreamSynchronize(r->down));
  return EJ_OK;
}

ej_status sj_resources(ej_handle* h, ej_stream_res** out) {
  if (!h->sres) {
    h->sres = new ej_stream_res();
    ej_stream_res* r = h->sres;
    EJ_CUDA(h, cudaStreamCreateWithFlags(&r->up, cudaStreamNonBlocking));
    EJ_CUDA(h, cudaStreamCreateWithFlags(&r->down, cudaStreamNonBlocking));
    for (cudaEvent_t& e : r->ev) EJ_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  *out = h->sres;
  return EJ_OK;
}

ej_status sj_device(ej_handle* h, ej_stream_res* r, size_t bytes) {
  if (bytes <= r->dev_cap) return EJ_OK;
  EJ_TRY(sj_idle(h, r));
  EJ_CUDA(h, cudaFree(r->dev));
  r->dev = nullptr;
  r->dev_cap = 0;
  if (ej_dev_alloc(&r->dev, bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    return ej_fail(h, EJ_ERR_NOMEM, "chunk buffers of %zu bytes could not be allocated", bytes);
  }
  r->dev_cap = bytes;
  return EJ_OK;
}

ej_status sj_rowbuf(ej_handle* h, ej_stream_res* r, uint64_t rows) {
  if (rows <= r->obuf_rows) return EJ_OK;
  rows = std::max<uint64_t>(rows + (rows >> 2), (uint64_t)1 << 20);
  EJ_TRY(sj_idle(h, r));
  EJ_CUDA(h, cudaFree(r->obuf));
  r->obuf = nullptr;
  r->obuf_rows = 0;
  if (ej_dev_alloc(&r->obuf, 2 * rows * sizeof(ej_result)) != cudaSuccess) {
    (void)cudaGetLastError();
    return ej_fail(h, EJ_ERR_NOMEM, "row buffers of %llu rows could not be allocated", (unsigned long long)rows);
  }
  r->obuf_rows = rows;
  return EJ_OK;
}

ej_status sj_bounce(ej_handle* h, ej_stream_res* r) {
  if (r->pin_cap) return EJ_OK;
  for (int i = 0; i < 2; i++)
    if (ej_host_alloc(&r->pin[i], SJ_BOUNCE) != cudaSuccess) {
      (void)cudaGetLastError();
      return ej_fail(h, EJ_ERR_NOMEM, "pinned bounce buffer of %zu bytes", SJ_BOUNCE);
    }
  r->pin_cap = SJ_BOUNCE;
  return EJ_OK;
}

// host-to-device copy of n tuples on the upload stream; pageable sources go
// through the bounce buffers (host memcpy, then a DMA copy)
ej_status sj_upload(ej_handle* h, ej_stream_res* r, ej_tuple* dst, const ej_tuple* src, uint64_t n, bool pinned,
                    int* turn) {
  const size_t bytes = n * sizeof(ej_tuple);
  if (pinned) {
    EJ_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, r->up));
    return EJ_OK;
  }
  for (size_t off = 0; off < bytes; off += r->pin_cap) {
    const size_t len = std::min(r->pin_cap, bytes - off);
    const int b = *turn;
    *turn ^= 1;
    EJ_CUDA(h, cudaEventSynchronize(r->ev[SR_PIN_FREE + b]));  // its previous copy has finished
    memcpy(r->pin[b], reinterpret_cast<const char*>(src) + off, len);
    EJ_CUDA(h, cudaMemcpyAsync(reinterpret_cast<char*>(dst) + off, r->pin[b], len, cudaMemcpyHostToDevice, r->up));
    EJ_CUDA(h, cudaEventRecord(r->ev[SR_PIN_FREE + b], r->up));
  }
  return EJ_OK;
}

// one device word read back on the compute stream (waits for it)
ej_status sj_read_word(ej_handle* h, ej_stream_res* r, const unsigned long long* d, uint64_t* v) {
  EJ_CUDA(h, cudaMemcpyAsync(h->h_words + 1, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  EJ_CUDA(h, cudaEventRecord(r->ev[SR_COUNT], h->stream));
  EJ_CUDA(h, cudaEventSynchronize(r->ev[SR_COUNT]));
  *v = h->h_words[1];
  return EJ_OK;
}

struct Job {
  ej_algo algo;
  ej_result* out;     // host rows
  ej_result* mapped;  // device view of a pinned out, or nullptr
  uint64_t cap;
  uint64_t total = 0;  // rows counted so far (hash join and the pageable-out nested loop)
  // hash join of the current R block
  ej_table_view t{};
  size_t probe_base = 0;
  uint32_t pb = 0;
};

// rows [total, total + w) of the result are in device buffer b: download them
ej_status sj_download(ej_handle* h, ej_stream_res* r, Job& j, int b, uint64_t w) {
  ej_result* src = reinterpret_cast<ej_result*>(r->obuf) + (size_t)b * r->obuf_rows;
  EJ_CUDA(h, cudaEventRecord(r->ev[SR_O_READY + b], h->stream));
  EJ_CUDA(h, cudaStreamWaitEvent(r->down, r->ev[SR_O_READY + b], 0));
  EJ_CUDA(h, cudaMemcpyAsync(j.out + j.total, src, w * sizeof(ej_result), cudaMemcpyDeviceToHost, r->down));
  EJ_CUDA(h, cudaEventRecord(r->ev[SR_O_FREE + b], r->down));
  return EJ_OK;
}

// hash join of one S chunk against the current block's table, in two halves:
// begin enqueues [partition +] count and the read-back of the count, finish
// waits for it and writes the rows (the next chunk is staged in between)
struct HashChunk {
  ej_probe_layout L;
  const ej_tuple* P = nullptr;
};

ej_status sj_hash_begin(ej_handle* h, ej_stream_res* r, Job& j, const ej_tuple* Sd, uint64_t n, HashChunk& c) {
  ej_plan_bytes p;
  p.bytes = j.probe_base;
  ej_probe_layout_add(p, c.L, n, j.pb, false, true);  // within the space reserved for a full chunk
  if (p.bytes > h->arena_cap) return ej_fail(h, EJ_ERR_INTERNAL, "chunk probe layout exceeds its reservation");
  c.P = Sd;
  if (c.L.pb) {
    ej_tuple* spart = reinterpret_cast<ej_tuple*>(ej_arena_at(h, c.L.spart_off));
    EJ_TRY(ej_partition_pass(h, c.L.splan, Sd, spart, 32u - c.L.pb, c.L.pb));
    c.P = spart;
  }
  EJ_TRY(ej_probe_count(h, c.L.pp, c.P, j.t, false, h->d_words + 1));
  EJ_CUDA(h, cudaMemcpyAsync(h->h_words + 1, h->d_words + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             h->stream));
  EJ_CUDA(h, cudaEventRecord(r->ev[SR_COUNT], h->stream));
  return EJ_OK;
}

ej_status sj_hash_finish(ej_handle* h, ej_stream_res* r, Job& j, int b, const HashChunk& c) {
  EJ_CUDA(h, cudaEventSynchronize(r->ev[SR_COUNT]));
  const uint64_t cnt = h->h_words[1];
  const uint64_t w = j.total < j.cap ? std::min(cnt, j.cap - j.total) : 0;
  if (w) {
    if (j.mapped) {
      EJ_TRY(ej_probe_write(h, c.L.pp, c.P, j.t, j.mapped + j.total, w));
    } else {
      EJ_TRY(sj_rowbuf(h, r, w));
      EJ_CUDA(h, cudaStreamWaitEvent(h->stream, r->ev[SR_O_FREE + b], 0));
      EJ_TRY(ej_probe_write(h, c.L.pp, c.P, j.t,
                            reinterpret_cast<ej_result*>(r->obuf) + (size_t)b * r->obuf_rows, w));
      EJ_TRY(sj_download(h, r, j, b, w));
    }
  }
  j.total += cnt;
  return EJ_OK;
}

// block nested loop of one S chunk against the current R block, in the same
// two halves; with a pinned out the rows go straight there (the cursor runs
// over the whole call) and finish has nothing to do
ej_status sj_bnl_begin(ej_handle* h, ej_stream_res* r, Job& j, int b, const ej_tuple* Rd, uint64_t nb,
                       const ej_tuple* Sd, uint64_t n) {
  if (j.mapped) return ej_bnl_append(h, Rd, nb, Sd, n, j.mapped, j.cap, h->d_words + 2);
  const uint64_t room = j.total < j.cap ? j.cap - j.total : 0;
  EJ_CUDA(h, cudaMemsetAsync(h->d_words + 1, 0, sizeof(unsigned long long), h->stream));
  EJ_CUDA(h, cudaStreamWaitEvent(h->stream, r->ev[SR_O_FREE + b], 0));
  ej_result* dst = r->obuf ? reinterpret_cast<ej_result*>(r->obuf) + (size_t)b * r->obuf_rows : nullptr;
  EJ_TRY(ej_bnl_append(h, Rd, nb, Sd, n, dst, std::min(room, r->obuf_rows), h->d_words + 1));
  EJ_CUDA(h, cudaMemcpyAsync(h->h_words + 1, h->d_words + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             h->stream));
  EJ_CUDA(h, cudaEventRecord(r->ev[SR_COUNT], h->stream));
  return EJ_OK;
}

ej_status sj_bnl_finish(ej_handle* h, ej_stream_res* r, Job& j, int b, const ej_tuple* Rd, uint64_t nb,
                        const ej_tuple* Sd, uint64_t n) {
  if (j.mapped) return EJ_OK;
  const uint64_t room = j.total < j.cap ? j.cap - j.total : 0;
  EJ_CUDA(h, cudaEventSynchronize(r->ev[SR_COUNT]));
  uint64_t cnt = h->h_words[1];
  const uint64_t w = std::min(cnt, room);
  if (w > r->obuf_rows) {  // more rows than the buffer holds: grow it and run the chunk again
    EJ_TRY(sj_rowbuf(h, r, w));
    EJ_CUDA(h, cudaMemsetAsync(h->d_words + 1, 0, sizeof(unsigned long long), h->stream));
    EJ_TRY(ej_bnl_append(h, Rd, nb, Sd, n, reinterpret_cast<ej_result*>(r->obuf) + (size_t)b * r->obuf_rows, w,
                         h->d_words + 1));
    EJ_TRY(sj_read_word(h, r, h->d_words + 1, &cnt));
  }
  if (w) EJ_TRY(sj_download(h, r, j, b, w));
  j.total += cnt;
  return EJ_OK;
}

uint64_t sj_default_block(ej_handle* h, uint64_t nR, uint64_t s_chunk) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    (void)cudaGetLastError();
    free_b = (size_t)8 << 30;
  }
  // per R row: the copy, the table and its build buffers (about 48 bytes);
  // per S row of a chunk: two buffers, the partitioned copy and the probe scratch (about 48 bytes)
  const double budget = 0.5 * (double)(free_b + h->arena_cap) - 48.0 * (double)s_chunk;
  const uint64_t rows = budget > 0 ? (uint64_t)(budget / 48.0) : 0;
  return std::max<uint64_t>(std::min<uint64_t>(std::min(nR, rows), (uint64_t)1 << 31), 1);
}

}  // namespace

extern "C" ej_status ej_join_host_chunked(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR,
                                          const ej_tuple* S, uint64_t nS, ej_result* out, uint64_t out_cap,
                                          uint64_t* out_count, const ej_chunk_config* cfg) {
  EJ_TRY(ej_begin(h));
  if ((nR && !R) || (nS && !S) || (out_cap && !out) || !out_count) return ej_fail(h, EJ_ERR_INVALID, "null buffer");
  if (algo != EJ_ALGO_HASH && algo != EJ_ALGO_BNL)
    return ej_fail(h, EJ_ERR_INVALID, "the chunked path runs the hash join and the block nested loop");
  *out_count = 0;
  if (nR == 0 || nS == 0) return EJ_OK;
  uint64_t s_chunk = cfg && cfg->s_chunk_rows ? cfg->s_chunk_rows : SJ_DEFAULT_CHUNK;
  s_chunk = std::min(std::min(s_chunk, nS), SJ_MAX_ROWS);
  uint64_t r_block = cfg && cfg->r_block_rows ? cfg->r_block_rows : sj_default_block(h, nR, s_chunk);
  r_block = std::min(std::min(r_block, nR), SJ_MAX_ROWS);

  ej_stream_res* r = nullptr;
  EJ_TRY(sj_resources(h, &r));
  const bool r_pinned = sj_pinned(R), s_pinned = sj_pinned(S);
  if (!r_pinned || !s_pinned) EJ_TRY(sj_bounce(h, r));
  Job j;
  j.algo = algo;
  j.out = out;
  j.cap = out_cap;
  j.mapped = out_cap ? static_cast<ej_result*>(sj_mapped(out)) : nullptr;
  if (j.mapped && reinterpret_cast<uintptr_t>(j.mapped) % 16) j.mapped = nullptr;
  if (!j.mapped && out_cap) EJ_TRY(sj_rowbuf(h, r, std::min(out_cap, s_chunk)));

  ej_plan_bytes dp;
  const size_t r_off = dp.add(r_block * sizeof(ej_tuple));
  const size_t s_off[2] = {dp.add(s_chunk * sizeof(ej_tuple)), dp.add(s_chunk * sizeof(ej_tuple))};
  EJ_TRY(sj_device(h, r, dp.bytes));
  char* dbase = static_cast<char*>(r->dev);
  ej_tuple* dR = reinterpret_cast<ej_tuple*>(dbase + r_off);
  ej_tuple* dS[2] = {reinterpret_cast<ej_tuple*>(dbase + s_off[0]), reinterpret_cast<ej_tuple*>(dbase + s_off[1])};
  EJ_CUDA(h, cudaMemsetAsync(h->d_words + 2, 0, sizeof(unsigned long long), h->stream));

  int turn = 0;
  const uint64_t nc = (nS + s_chunk - 1) / s_chunk;
  for (uint64_t r0 = 0; r0 < nR; r0 += r_block) {
    const uint64_t nb = std::min(r_block, nR - r0);
    // the previous block's chunks are done with dR and the S buffers
    EJ_CUDA(h, cudaEventRecord(r->ev[SR_BLOCK_DONE], h->stream));
    EJ_CUDA(h, cudaStreamWaitEvent(r->up, r->ev[SR_BLOCK_DONE], 0));
    EJ_TRY(sj_upload(h, r, dR, R + r0, nb, r_pinned, &turn));
    EJ_CUDA(h, cudaEventRecord(r->ev[SR_R_READY], r->up));
    EJ_CUDA(h, cudaStreamWaitEvent(h->stream, r->ev[SR_R_READY], 0));
    if (algo == EJ_ALGO_HASH) {
      ej_plan_bytes p;
      ej_table_plan_t tp;
      ej_table_plan(p, tp, nb, /*own_storage=*/false, EJ_TABLE_HASH, ej_tuned_table_knobs(h, nb), nS);
      j.probe_base = p.bytes;
      j.pb = ej_probe_partition_bits(h, nb, s_chunk);
      ej_probe_layout L;
      ej_probe_layout_add(p, L, s_chunk, j.pb, false, true);
      EJ_TRY(ej_arena_reserve(h, p.bytes));
      EJ_TRY(ej_table_build(h, tp, dR, reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rkey_off)),
                            reinterpret_cast<int32_t*>(ej_arena_at(h, tp.rval_off)), ej_arena_at(h, tp.aux_off),
                            &j.t));
    }
    // S chunk i+1 uploads while chunk i joins
    auto issue = [&](uint64_t i) -> ej_status {
      const int b = (int)(i & 1);
      const uint64_t s0 = i * s_chunk, n = std::min(s_chunk, nS - s0);
      EJ_CUDA(h, cudaStreamWaitEvent(r->up, r->ev[SR_S_FREE + b], 0));
      EJ_TRY(sj_upload(h, r, dS[b], S + s0, n, s_pinned, &turn));
      EJ_CUDA(h, cudaEventRecord(r->ev[SR_S_READY + b], r->up));
      return EJ_OK;
    };
    EJ_TRY(issue(0));
    for (uint64_t i = 0; i < nc; i++) {
      const int b = (int)(i & 1);
      const uint64_t n = std::min(s_chunk, nS - i * s_chunk);
      EJ_CUDA(h, cudaStreamWaitEvent(h->stream, r->ev[SR_S_READY + b], 0));
      HashChunk c;
      if (algo == EJ_ALGO_HASH)
        EJ_TRY(sj_hash_begin(h, r, j, dS[b], n, c));
      else
        EJ_TRY(sj_bnl_begin(h, r, j, b, dR, nb, dS[b], n));
      if (i + 1 < nc) EJ_TRY(issue(i + 1));  // staged while chunk i runs
      if (algo == EJ_ALGO_HASH)
        EJ_TRY(sj_hash_finish(h, r, j, b, c));
      else
        EJ_TRY(sj_bnl_finish(h, r, j, b, dR, nb, dS[b], n));
      EJ_CUDA(h, cudaEventRecord(r->ev[SR_S_FREE + b], h->stream));
    }
  }
  EJ_TRY(sj_idle(h, r));
  uint64_t total = j.total;
  if (algo == EJ_ALGO_BNL && j.mapped) {
    EJ_TRY(sj_read_word(h, r, h->d_words + 2, &total));
  }
  // device status: a bounded wait that gave up, or rows past a capacity
  EJ_TRY(ej_finish(h, nullptr));
  *out_count = total;
  return ej_capacity_result(h, total, out_cap);
}
