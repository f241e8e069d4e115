"""ctypes wrapper of the C oracle (oracle/ej_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the bench's
CPU-baseline leg as the checker.  The join engine never imports this module.
Arrays are numpy int32: relations (n, 2) = TUPLE{key, val}, results (n, 4) =
RESULT{rkey, rval, lkey, lval}, star results (n, 8).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(ORACLE_DIR)
LIB = os.path.join(ORACLE_DIR, "_build", "libej_oracle.so")
SRC = os.path.join(ORACLE_DIR, "ej_oracle.c")
GEN_H = os.path.join(ROOT, "include", "ej_gen.h")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(p) for p in (SRC, GEN_H)):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I",
           os.path.join(ROOT, "include"), SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        vp, u64, u32 = C.c_void_p, C.c_uint64, C.c_uint32
        for name in ("ejo_hash_join", "ejo_hash_index_join", "ejo_left_outer_join"):
            getattr(lib, name).argtypes = [vp, u64, vp, u64, vp, u64, u32]
            getattr(lib, name).restype = u64
        for name in ("ejo_sort_index_join", "ejo_bnl_join"):
            getattr(lib, name).argtypes = [vp, u64, vp, u64, vp, u64]
            getattr(lib, name).restype = u64
        lib.ejo_hash_join_mt.argtypes = [vp, u64, vp, u64, vp, u64, u32, u32]
        lib.ejo_hash_join_mt.restype = u64
        lib.ejo_hash_join_count.argtypes = [vp, u64, vp, u64, u32]
        lib.ejo_hash_join_count.restype = u64
        lib.ejo_star_join3.argtypes = [vp, vp, u64, vp, u64, vp, u64, vp, u64, u32]
        lib.ejo_star_join3.restype = u64
        lib.ejo_generate.argtypes = [vp, vp]
        lib.ejo_zipf_cdf.argtypes = [C.c_double, u32, vp]
        lib.ejo_canon_sort.argtypes = [vp, u64]
        lib.ejo_canon_sort_star.argtypes = [vp, u64]
        lib.ejo_checksum.argtypes = [vp, u64, u32]
        lib.ejo_checksum.restype = u64
        _lib = lib
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None or a.size == 0 else a.ctypes.data


def _rel(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.int32)
    assert a.ndim == 2 and a.shape[1] == 2
    return a


def generate(spec) -> np.ndarray:
    """Host copy of a generated relation (same generator as the device).

    Zipf specs with s > 0 get their CDF table built here (ejo_zipf_cdf)."""
    lib = load()
    out = np.empty((spec.n, 2), dtype=np.int32)
    keep = None
    if spec.kind == 2 and spec.zipf_s != 0.0 and not spec.cdf:
        keep = np.empty(spec.domain, dtype=np.float64)
        lib.ejo_zipf_cdf(spec.zipf_s, spec.domain, keep.ctypes.data)
        spec.cdf = keep.ctypes.data
    try:
        if spec.n:
            lib.ejo_generate(C.byref(spec), out.ctypes.data)
    finally:
        if keep is not None:
            spec.cdf = None
    return out


def _join(name: str, R, S, extra=()) -> np.ndarray:
    lib = load()
    R, S = _rel(R), _rel(S)
    fn = getattr(lib, name)
    n = fn(_p(R), len(R), _p(S), len(S), None, 0, *extra)
    if n == 2 ** 64 - 1:
        raise MemoryError(name)
    out = np.empty((n, 4), dtype=np.int32)
    m = fn(_p(R), len(R), _p(S), len(S), _p(out), n, *extra)
    assert m == n
    return out


def hash_join(R, S, nb_bktent: int = 1 << 20) -> np.ndarray:
    """joins/CPU_JOIN/hash_cpu restated (partitioned hash join)."""
    return _join("ejo_hash_join", R, S, (nb_bktent,))


def hash_join_mt(R, S, threads: int = 0, partitions: int = 1 << 17) -> np.ndarray:
    """joins/multi_joins/hash restated (pthread partitioned hash join); threads 0: every host core."""
    lib = load()
    R, S = _rel(R), _rel(S)
    nt = threads or os.cpu_count() or 8
    n = int(lib.ejo_hash_join_mt(_p(R), len(R), _p(S), len(S), None, 0, partitions, nt))
    out = np.empty((max(n, 1), 4), dtype=np.int32)
    m = int(lib.ejo_hash_join_mt(_p(R), len(R), _p(S), len(S), _p(out), n, partitions, nt))
    if m == 2 ** 64 - 1:
        raise MemoryError("ejo_hash_join_mt")
    assert m == n
    return out[:n]


def hash_index_join(R, S, nb_bucket: int = 1 << 20) -> np.ndarray:
    """joins/CPU_JOIN/inner_cpu restated (hash-index join; NB_BUCKET is 2^27 there)."""
    return _join("ejo_hash_index_join", R, S, (nb_bucket,))


def sort_index_join(R, S) -> np.ndarray:
    """joins/CPU_JOIN/sortIndex_cpu restated (quicksort index + binary search)."""
    return _join("ejo_sort_index_join", R, S)


def bnl_join(R, S) -> np.ndarray:
    """joins/CPU_JOIN/block_cpu restated (nested loop over all pairs)."""
    return _join("ejo_bnl_join", R, S)


def left_outer_join(R, S, nb_bucket: int = 1 << 20) -> np.ndarray:
    """Inner hash-index join plus (INT32_MIN, INT32_MIN, s.key, s.val) per unmatched S row."""
    return _join("ejo_left_outer_join", R, S, (nb_bucket,))


def hash_join_count(R, S, nb_bucket: int = 1 << 20) -> int:
    lib = load()
    R, S = _rel(R), _rel(S)
    return int(lib.ejo_hash_join_count(_p(R), len(R), _p(S), len(S), nb_bucket))


def star_join3(F1, F2, D1, D2, nb_bucket: int = 1 << 20) -> np.ndarray:
    lib = load()
    F1, F2, D1, D2 = (_rel(x) for x in (F1, F2, D1, D2))
    args = (_p(F1), _p(F2), len(F1), _p(D1), len(D1), _p(D2), len(D2))
    n = lib.ejo_star_join3(*args, None, 0, nb_bucket)
    out = np.empty((n, 8), dtype=np.int32)
    lib.ejo_star_join3(*args, _p(out), n, nb_bucket)
    return out


def canon(rows: np.ndarray) -> np.ndarray:
    """Canonical order: lexicographic over the signed int32 columns."""
    rows = np.ascontiguousarray(rows, dtype=np.int32).copy()
    lib = load()
    if len(rows):
        if rows.shape[1] == 4:
            lib.ejo_canon_sort(rows.ctypes.data, len(rows))
        else:
            lib.ejo_canon_sort_star(rows.ctypes.data, len(rows))
    return rows


def checksum(rows: np.ndarray) -> int:
    """Order-independent 64-bit checksum (sum of a per-row mix), as ej_checksum computes."""
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    return int(load().ejo_checksum(_p(rows), len(rows), rows.shape[1] if rows.ndim == 2 else 4))
