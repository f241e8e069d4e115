// table_file.cu - the reference's on-disk relation formats (host code).
//
//   EJ_TABLE_FILE_COUNTED  a 4-byte count n, then n 8-byte tuples: written by
//                          joins/hashJoin_gpu/main_street/TableBuild.cpp:113-140
//                          and read back by joins/hashJoin_gpu/disk_hash/hj.cc:212-266;
//   EJ_TABLE_FILE_RAW      tuples only, n = file size / 8: the joins/join_ori R
//                          and S files, read by joins/join_ori/hj.cc:68-78.
//
// Loading into device memory streams the file through two pinned buffers: the
// read of chunk i + 1 overlaps the host-to-device copy of chunk i on the
// handle's stream.  Saving from device memory overlaps the same way in the
// other direction.  Both formats are little-endian, as on the reference's x86
// hosts and on every host this library builds for.
#include <stdio.h>

#include <algorithm>

#include "ej_entry.h"
#include "ej_internal.h"

namespace {

constexpr size_t TF_CHUNK = (size_t)32 << 20;  // bytes per staging buffer

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

// host-side failure without a handle: the status alone
ej_status tf_open(const char* path, const char* mode, File& file) {
  if (!path) return EJ_ERR_INVALID;
  file.f = fopen(path, mode);
  return file.f ? EJ_OK : EJ_ERR_IO;
}

// rows of an open table file, leaving the stream at the first tuple
ej_status tf_rows(File& file, ej_table_file_format fmt, uint64_t* n) {
  if (fmt == EJ_TABLE_FILE_COUNTED) {
    int32_t c = 0;
    if (fread(&c, sizeof c, 1, file.f) != 1 || c < 0) return EJ_ERR_IO;
    // the file must hold every tuple the header announces
    const long here = ftell(file.f);
    if (fseek(file.f, 0, SEEK_END) != 0) return EJ_ERR_IO;
    const long size = ftell(file.f);
    if (here < 0 || size < 0 || fseek(file.f, here, SEEK_SET) != 0) return EJ_ERR_IO;
    if ((uint64_t)(size - here) < (uint64_t)c * sizeof(ej_tuple)) return EJ_ERR_IO;
    *n = (uint64_t)c;
    return EJ_OK;
  }
  if (fmt == EJ_TABLE_FILE_RAW) {
    if (fseek(file.f, 0, SEEK_END) != 0) return EJ_ERR_IO;
    const long size = ftell(file.f);
    if (size < 0 || size % (long)sizeof(ej_tuple) != 0 || fseek(file.f, 0, SEEK_SET) != 0) return EJ_ERR_IO;
    *n = (uint64_t)size / sizeof(ej_tuple);
    return EJ_OK;
  }
  return EJ_ERR_INVALID;
}

struct Pinned {
  void* p[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~Pinned() {
    for (int i = 0; i < 2; i++) {
      if (ev[i]) cudaEventDestroy(ev[i]);
      if (p[i]) cudaFreeHost(p[i]);
    }
  }
};

ej_status tf_pinned(ej_handle* h, Pinned& pin) {
  for (int i = 0; i < 2; i++) {
    if (ej_host_alloc(&pin.p[i], TF_CHUNK) != cudaSuccess) {
      (void)cudaGetLastError();
      return ej_fail(h, EJ_ERR_NOMEM, "pinned staging buffer of %zu bytes", TF_CHUNK);
    }
    EJ_CUDA(h, cudaEventCreateWithFlags(&pin.ev[i], cudaEventDisableTiming));
  }
  return EJ_OK;
}

bool tf_is_device(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" ej_status ej_table_file_rows(const char* path, ej_table_file_format fmt, uint64_t* n) {
  if (!n) return EJ_ERR_INVALID;
  File file;
  ej_status s = tf_open(path, "rb", file);
  if (s != EJ_OK) return s;
  return tf_rows(file, fmt, n);
}

extern "C" ej_status ej_table_file_read(const char* path, ej_table_file_format fmt, ej_tuple* dst, uint64_t cap,
                                        uint64_t* n) {
  if (!n) return EJ_ERR_INVALID;
  File file;
  ej_status s = tf_open(path, "rb", file);
  if (s != EJ_OK) return s;
  if ((s = tf_rows(file, fmt, n)) != EJ_OK) return s;
  if (*n > cap) return EJ_ERR_CAPACITY;
  if (*n && !dst) return EJ_ERR_INVALID;
  return fread(dst, sizeof(ej_tuple), (size_t)*n, file.f) == (size_t)*n ? EJ_OK : EJ_ERR_IO;
}

extern "C" ej_status ej_table_load(ej_handle* h, const char* path, ej_table_file_format fmt, ej_tuple* dst,
                                   uint64_t cap, uint64_t* n) {
  EJ_TRY(ej_begin(h));
  if (!n) return ej_fail(h, EJ_ERR_INVALID, "n is NULL");
  File file;
  if (tf_open(path, "rb", file) != EJ_OK) return ej_fail(h, EJ_ERR_IO, "cannot open %s", path ? path : "(null)");
  if (tf_rows(file, fmt, n) != EJ_OK) return ej_fail(h, EJ_ERR_IO, "%s is not a table file of that format", path);
  if (*n > cap) return ej_fail(h, EJ_ERR_CAPACITY, "%s holds %llu rows, capacity %llu", path,
                               (unsigned long long)*n, (unsigned long long)cap);
  if (*n == 0) return EJ_OK;
  EJ_TRY(ej_check_rel(h, "dst", dst, *n));
  Pinned pin;
  EJ_TRY(tf_pinned(h, pin));
  const uint64_t bytes = *n * sizeof(ej_tuple);
  char* d = reinterpret_cast<char*>(dst);
  int b = 0;
  for (uint64_t off = 0; off < bytes; off += TF_CHUNK, b ^= 1) {
    const size_t len = (size_t)std::min<uint64_t>(TF_CHUNK, bytes - off);
    EJ_CUDA(h, cudaEventSynchronize(pin.ev[b]));  // the copy out of this buffer has finished
    if (fread(pin.p[b], 1, len, file.f) != len) {
      (void)cudaStreamSynchronize(h->stream);
      return ej_fail(h, EJ_ERR_IO, "short read of %s", path);
    }
    EJ_CUDA(h, cudaMemcpyAsync(d + off, pin.p[b], len, cudaMemcpyHostToDevice, h->stream));
    EJ_CUDA(h, cudaEventRecord(pin.ev[b], h->stream));
  }
  EJ_CUDA(h, cudaStreamSynchronize(h->stream));  // the staging buffers die with this call
  return EJ_OK;
}

extern "C" ej_status ej_table_save(ej_handle* h, const char* path, ej_table_file_format fmt, const ej_tuple* src,
                                   uint64_t n) {
  EJ_TRY(ej_begin(h));
  if (fmt != EJ_TABLE_FILE_COUNTED && fmt != EJ_TABLE_FILE_RAW) return ej_fail(h, EJ_ERR_INVALID, "bad format");
  if (fmt == EJ_TABLE_FILE_COUNTED && n > (uint64_t)INT32_MAX)
    return ej_fail(h, EJ_ERR_TOO_LARGE, "the counted format holds at most 2^31 - 1 rows");
  if (n && !src) return ej_fail(h, EJ_ERR_INVALID, "src is NULL");
  File file;
  if (tf_open(path, "wb", file) != EJ_OK) return ej_fail(h, EJ_ERR_IO, "cannot create %s", path ? path : "(null)");
  if (fmt == EJ_TABLE_FILE_COUNTED) {
    const int32_t c = (int32_t)n;
    if (fwrite(&c, sizeof c, 1, file.f) != 1) return ej_fail(h, EJ_ERR_IO, "write to %s failed", path);
  }
  const uint64_t bytes = n * sizeof(ej_tuple);
  if (n && !tf_is_device(src)) {
    if (fwrite(src, 1, (size_t)bytes, file.f) != (size_t)bytes) return ej_fail(h, EJ_ERR_IO, "write to %s failed", path);
    return EJ_OK;
  }
  Pinned pin;
  if (n) EJ_TRY(tf_pinned(h, pin));
  const char* s = reinterpret_cast<const char*>(src);
  // copy chunk i + 1 while chunk i is written to the file
  size_t pending_len = 0;
  int b = 0;
  for (uint64_t off = 0; off < bytes; off += TF_CHUNK, b ^= 1) {
    const size_t len = (size_t)std::min<uint64_t>(TF_CHUNK, bytes - off);
    EJ_CUDA(h, cudaMemcpyAsync(pin.p[b], s + off, len, cudaMemcpyDeviceToHost, h->stream));
    EJ_CUDA(h, cudaEventRecord(pin.ev[b], h->stream));
    if (pending_len) {
      EJ_CUDA(h, cudaEventSynchronize(pin.ev[b ^ 1]));
      if (fwrite(pin.p[b ^ 1], 1, pending_len, file.f) != pending_len) {
        (void)cudaStreamSynchronize(h->stream);
        return ej_fail(h, EJ_ERR_IO, "write to %s failed", path);
      }
    }
    pending_len = len;
  }
  if (pending_len) {
    EJ_CUDA(h, cudaEventSynchronize(pin.ev[b ^ 1]));
    if (fwrite(pin.p[b ^ 1], 1, pending_len, file.f) != pending_len)
      return ej_fail(h, EJ_ERR_IO, "write to %s failed", path);
  }
  return fflush(file.f) == 0 ? EJ_OK : ej_fail(h, EJ_ERR_IO, "write to %s failed", path);
}
