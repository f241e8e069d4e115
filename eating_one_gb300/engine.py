"""Python mirror of the C ABI over torch device tensors.

Relations are int32 tensors of shape (n, 2) holding TUPLE{key, val} rows;
results are int32 tensors of shape (n, 4) holding RESULT{rkey, rval, lkey,
lval} rows (star join: (n, 8)).  Every call goes through libeating_one.so;
there is no other implementation of any join.
"""
from __future__ import annotations

import ctypes as C
import os

import torch

from . import native
from .native import GenSpec


class JoinError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (native.load().ej_status_name(status).decode(), message))
        self.status = status


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None or t.numel() == 0 else t.data_ptr()


class Index:
    """A device-resident hash or sort index on R (ej_index)."""

    def __init__(self, engine: "Engine", handle: C.c_void_p, kind: str, R: torch.Tensor):
        self.engine, self.handle, self.kind, self.R = engine, handle, kind, R

    def join(self, S: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        return self.engine._run_sized(lambda o, cap, cnt: self.engine.lib.ej_index_join(
            self.engine.h, self.handle, _ptr(S), S.shape[0], o, cap, cnt), out, 4)

    def left_outer_join(self, S: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        return self.engine._run_sized(lambda o, cap, cnt: self.engine.lib.ej_index_left_outer_join(
            self.engine.h, self.handle, _ptr(S), S.shape[0], o, cap, cnt), out, 4)

    def merge_join(self, S: torch.Tensor, s_sorted: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
        """Merge join with S in value order (sort indexes; s_sorted False: the call sorts a copy of S)."""
        if out is None:
            out = torch.empty((self.count(S), 4), dtype=torch.int32, device=self.engine.device)
        return self.engine._run_sized(lambda o, cap, cnt: self.engine.lib.ej_index_merge_join(
            self.engine.h, self.handle, _ptr(S), S.shape[0], 1 if s_sorted else 0, o, cap, cnt), out, 4)

    def count(self, S: torch.Tensor) -> int:
        cnt = C.c_uint64(0)
        self.engine._check(self.engine.lib.ej_index_join_count(
            self.engine.h, self.handle, _ptr(S), S.shape[0], C.byref(cnt)))
        return cnt.value

    def free(self) -> None:
        if self.handle:
            self.engine._check(self.engine.lib.ej_index_free(self.engine.h, self.handle))
            self.handle = None


class Engine:
    """One ej_handle bound to one CUDA device."""

    def __init__(self, device: int = 0, tuned: bool = True):
        """tuned: install the tuning table measured on GB300
        (eating_one_gb300/tuning_gb300.json, autotune.py) when it exists."""
        self.lib = native.load()
        self.device = torch.device("cuda", device)
        h = C.c_void_p()
        st = self.lib.ej_create(device, C.byref(h))
        if st != native.EJ_OK:
            raise JoinError(st, "ej_create(%d) failed" % device)
        self.h = h
        if tuned:
            from . import autotune
            autotune.load_default(self)

    # ---- plumbing -------------------------------------------------------------
    def close(self) -> None:
        if self.h:
            self.lib.ej_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self.lib.ej_last_error(self.h).decode()

    def _check(self, st: int, allow_capacity: bool = False) -> int:
        if st == native.EJ_OK or (allow_capacity and st == native.EJ_ERR_CAPACITY):
            return st
        raise JoinError(st, self.last_error())

    def _sync_stream(self) -> None:
        self.lib.ej_set_stream(self.h, torch.cuda.current_stream(self.device).cuda_stream)

    def set_option(self, name: str, value: int) -> None:
        opt = {"partition_bits": 0, "bucket_bits_delta": 1, "wait_limit_ns": 2, "count_reuse": 3, "build": 4,
               "table": 5, "probe_warps": 6}[name]
        self._check(self.lib.ej_set_option(self.h, opt, value))

    def set_timing(self, enable: bool) -> None:
        self._check(self.lib.ej_set_timing(self.h, 1 if enable else 0))

    def phase_ms(self) -> list[float]:
        """Device time of the last timed join's phases: build, partition, count, write (ms)."""
        arr = (C.c_float * native.EJ_PHASES)()
        self._check(self.lib.ej_last_phase_ms(self.h, arr))
        return list(arr)

    def phase_totals(self) -> tuple[list[float], int]:
        """Summed phase times of every join timed since the last call, and how many joins."""
        arr = (C.c_double * native.EJ_PHASES)()
        n = C.c_uint32(0)
        self._check(self.lib.ej_phase_totals(self.h, arr, C.byref(n)))
        return list(arr), n.value

    def kernel_launches(self) -> int:
        return int(self.lib.ej_kernel_launches(self.h))

    def scratch_bytes(self) -> int:
        return int(self.lib.ej_scratch_bytes(self.h))

    def trim(self) -> None:
        self._check(self.lib.ej_trim(self.h))

    def _run_sized(self, call, out: torch.Tensor | None, width: int) -> torch.Tensor:
        """Run `call(out_ptr, cap, &count)`; size the output from the count when needed."""
        self._sync_stream()
        cnt = C.c_uint64(0)
        if out is None:
            st = self._check(call(None, 0, C.byref(cnt)), allow_capacity=True)
            out = torch.empty((cnt.value, width), dtype=torch.int32, device=self.device)
            if cnt.value == 0:
                return out
        st = self._check(call(_ptr(out), out.shape[0], C.byref(cnt)), allow_capacity=True)
        if st == native.EJ_ERR_CAPACITY:
            raise JoinError(st, "%d results do not fit the %d-row output" % (cnt.value, out.shape[0]))
        return out[: cnt.value]

    # ---- joins ------------------------------------------------------------------
    def join(self, algo: str, R: torch.Tensor, S: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        a = native.ALGO[algo]
        if out is None and algo == "hash":
            # the reference's sequence (hj.cc:997-1115): the count pass sizes the
            # output, then the join writes it; the handle keeps the count's table,
            # partitioned S and run descriptors, so the join only writes
            out = torch.empty((self.count("hash", R, S), 4), dtype=torch.int32, device=self.device)
            if out.shape[0] == 0:
                return out
        return self._run_sized(lambda o, cap, cnt: self.lib.ej_join(
            self.h, a, _ptr(R), R.shape[0], _ptr(S), S.shape[0], o, cap, cnt), out, 4)

    def hash_join(self, R, S, out=None):
        return self.join("hash", R, S, out)

    def count(self, algo: str, R: torch.Tensor, S: torch.Tensor) -> int:
        self._sync_stream()
        cnt = C.c_uint64(0)
        if algo == "hash":
            self._check(self.lib.ej_hash_join_count(self.h, _ptr(R), R.shape[0], _ptr(S), S.shape[0], C.byref(cnt)))
        elif algo == "bnl":
            self._check(self.lib.ej_bnl_join_count(self.h, _ptr(R), R.shape[0], _ptr(S), S.shape[0], C.byref(cnt)))
        else:
            self._check(self.lib.ej_join(self.h, native.ALGO[algo], _ptr(R), R.shape[0], _ptr(S), S.shape[0],
                                         None, 0, C.byref(cnt)), allow_capacity=True)
        return cnt.value

    def hash_join_async(self, R, S, out: torch.Tensor, d_count: torch.Tensor) -> None:
        """Asynchronous hash join: total count into d_count (int64[1]); rows past out's length dropped."""
        self._sync_stream()
        self._check(self.lib.ej_hash_join_async(self.h, _ptr(R), R.shape[0], _ptr(S), S.shape[0], _ptr(out),
                                                out.shape[0], d_count.data_ptr()))

    def sync_status(self) -> int:
        return self.lib.ej_sync_status(self.h)

    def batch_hash_join(self, pairs, outs=None) -> list[torch.Tensor]:
        """Hash-join many (R, S) pairs in one batched pipeline; returns each join's rows.

        outs: optional preallocated (cap, 4) tensors; without them each output is
        sized by its count (one count pass per join first)."""
        self._sync_stream()
        n = len(pairs)
        if outs is None:
            outs = [torch.empty((self.count("hash", R, S), 4), dtype=torch.int32, device=self.device)
                    for R, S in pairs]
        descs = (native.JoinDesc * max(n, 1))()
        for i, ((R, S), o) in enumerate(zip(pairs, outs)):
            descs[i].R, descs[i].nR = _ptr(R), R.shape[0]
            descs[i].S, descs[i].nS = _ptr(S), S.shape[0]
            descs[i].out, descs[i].out_cap = _ptr(o), o.shape[0]
        counts = (C.c_uint64 * max(n, 1))()
        self._check(self.lib.ej_batch_hash_join(self.h, descs, n, counts))
        return [o[: counts[i]] for i, o in enumerate(outs)]

    def batch_hash_join_async(self, descs, n: int, d_counts: torch.Tensor) -> None:
        """Asynchronous batch over prepared native.JoinDesc entries; counts to d_counts (int64[n])."""
        self._sync_stream()
        self._check(self.lib.ej_batch_hash_join_async(self.h, descs, n, d_counts.data_ptr()))

    def star_join3(self, F1, F2, D1, D2, out=None) -> torch.Tensor:
        return self._run_sized(lambda o, cap, cnt: self.lib.ej_star_join3(
            self.h, _ptr(F1), _ptr(F2), F1.shape[0], _ptr(D1), D1.shape[0], _ptr(D2), D2.shape[0], o, cap, cnt),
            out, 8)

    # ---- distance joins -------------------------------------------------------------
    def points_to_device(self, points) -> torch.Tensor:
        """A numpy array of native.point_dtype(dims) as a (n, point bytes) uint8 device tensor."""
        import numpy as np
        raw = np.ascontiguousarray(points).view(np.uint8).reshape(len(points), points.dtype.itemsize)
        return torch.from_numpy(raw).to(self.device)

    @staticmethod
    def rows_to_numpy(rows: torch.Tensor, dims: int):
        """Distance-join rows (uint8 tensor) as a numpy array of native.point_result_dtype(dims)."""
        return rows.cpu().contiguous().numpy().reshape(-1).view(native.point_result_dtype(dims))

    def distance_join(self, R: torch.Tensor, S: torch.Tensor, dims: int, radius: float = 1.0,
                      out: torch.Tensor | None = None) -> torch.Tensor:
        """Distance nested-loop join of device point arrays (see points_to_device): S point l
        and R point r match when sum_i (r.val[i] - l.val[i])^2 < radius^2.  Returns a
        (count, row bytes) uint8 tensor of native.point_result_dtype(dims) rows."""
        pb, rb = native.point_dtype(dims).itemsize, native.point_result_dtype(dims).itemsize
        nR, nS = R.numel() // pb, S.numel() // pb
        self._sync_stream()
        cnt = C.c_uint64(0)
        if out is None:
            self._check(self.lib.ej_distance_join_count(self.h, dims, _ptr(R), nR, _ptr(S), nS, radius,
                                                        C.byref(cnt)))
            out = torch.empty((cnt.value, rb), dtype=torch.uint8, device=self.device)
            if cnt.value == 0:
                return out
        st = self._check(self.lib.ej_distance_join(self.h, dims, _ptr(R), nR, _ptr(S), nS, radius, _ptr(out),
                                                   out.shape[0], C.byref(cnt)), allow_capacity=True)
        if st == native.EJ_ERR_CAPACITY:
            raise JoinError(st, "%d results do not fit the %d-row output" % (cnt.value, out.shape[0]))
        return out[: cnt.value]

    def distance_join_count(self, R: torch.Tensor, S: torch.Tensor, dims: int, radius: float = 1.0) -> int:
        pb = native.point_dtype(dims).itemsize
        self._sync_stream()
        cnt = C.c_uint64(0)
        self._check(self.lib.ej_distance_join_count(self.h, dims, _ptr(R), R.numel() // pb, _ptr(S),
                                                    S.numel() // pb, radius, C.byref(cnt)))
        return cnt.value

    def build_index(self, kind: str, R: torch.Tensor) -> Index:
        self._sync_stream()
        ix = C.c_void_p()
        fn = self.lib.ej_hash_index_build if kind == "hash" else self.lib.ej_sort_index_build
        self._check(fn(self.h, _ptr(R), R.shape[0], C.byref(ix)))
        return Index(self, ix, kind, R)

    def join_host(self, algo: str, R, S, out) -> int:
        """Host-buffer join (numpy or CPU tensors); returns the count (rows copied: min(count, len(out)))."""
        def p(a):
            return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()
        self._sync_stream()
        cnt = C.c_uint64(0)
        st = self.lib.ej_join_host(self.h, native.ALGO[algo], p(R), len(R), p(S), len(S), p(out), len(out),
                                   C.byref(cnt))
        self._check(st, allow_capacity=True)
        return cnt.value

    def join_host_chunked(self, algo: str, R, S, out, r_block: int = 0, s_chunk: int = 0) -> int:
        """Out-of-core host-buffer join ("hash" or "bnl"): R in device blocks of r_block rows, S
        streamed in chunks of s_chunk rows (0: sized by the library).  Returns the count; rows
        copied: min(count, len(out)).  Pinned host tensors are used in place."""
        def p(a):
            return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()
        self._sync_stream()
        cfg = native.ChunkConfig(r_block, s_chunk)
        cnt = C.c_uint64(0)
        st = self.lib.ej_join_host_chunked(self.h, native.ALGO[algo], p(R), len(R), p(S), len(S), p(out),
                                           len(out), C.byref(cnt), C.byref(cfg))
        self._check(st, allow_capacity=True)
        return cnt.value

    # ---- utilities ----------------------------------------------------------------
    def exclusive_scan_u32(self, x: torch.Tensor) -> torch.Tensor:
        self._sync_stream()
        out = torch.empty(x.numel() + 1, dtype=torch.int64, device=self.device)
        self._check(self.lib.ej_exclusive_scan_u32(self.h, _ptr(x), x.numel(), out.data_ptr()))
        return out

    def generate(self, spec: GenSpec) -> torch.Tensor:
        self._sync_stream()
        out = torch.empty((spec.n, 2), dtype=torch.int32, device=self.device)
        self._check(self.lib.ej_generate(self.h, C.byref(spec), _ptr(out)))
        return out

    def load_table(self, path: str, fmt: int = native.EJ_TABLE_FILE_COUNTED) -> torch.Tensor:
        """A table file (include/ej.h: EJ_TABLE_FILE_COUNTED or _RAW) as an (n, 2) int32 device tensor."""
        self._sync_stream()
        n = C.c_uint64(0)
        st = self.lib.ej_table_file_rows(os.fsencode(path), fmt, C.byref(n))
        if st != native.EJ_OK:
            raise JoinError(st, "cannot read %s as a table file" % path)
        out = torch.empty((max(n.value, 1), 2), dtype=torch.int32, device=self.device)[:n.value]
        self._check(self.lib.ej_table_load(self.h, os.fsencode(path), fmt, _ptr(out), n.value, C.byref(n)))
        return out

    def save_table(self, path: str, rows: torch.Tensor, fmt: int = native.EJ_TABLE_FILE_COUNTED) -> None:
        """Write an (n, 2) int32 relation (device or host) as a table file."""
        self._sync_stream()
        rows = rows.contiguous()
        self._check(self.lib.ej_table_save(self.h, os.fsencode(path), fmt, _ptr(rows), rows.shape[0]))

    def checksum(self, rows: torch.Tensor) -> int:
        """Order-independent checksum of result rows (same function as the oracle's)."""
        self._sync_stream()
        v = C.c_uint64(0)
        self._check(self.lib.ej_checksum(self.h, _ptr(rows), rows.shape[0], rows.shape[1], C.byref(v)))
        return v.value
