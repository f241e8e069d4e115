"""ctypes wrapper of the C oracle (oracle/ej_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the bench's
CPU-baseline leg as the checker.  The join engine never imports this module.
Arrays are numpy int32: relations (n, 2) = TUPLE{key, val}, results (n, 4) =
RESULT{rkey, rval, lkey, lval}, star results (n, 8).  Distance joins take and
return numpy structured arrays (POINT_DTYPE, POINT_RESULT_DTYPE).
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
        lib.ejo_distance_join.argtypes = [u32, vp, u64, vp, u64, C.c_double, vp, u64, u32]
        lib.ejo_distance_join.restype = u64
        pu64 = C.POINTER(u64)
        lib.ejo_join_digest_mt.argtypes = [vp, u64, vp, u64, C.c_int, u32, u32, pu64, pu64]
        lib.ejo_join_digest_mt.restype = C.c_int
        lib.ejo_star_digest_mt.argtypes = [vp, vp, u64, vp, u64, vp, u64, u32, u32, pu64, pu64]
        lib.ejo_star_digest_mt.restype = C.c_int
        lib.ejo_generate_mt.argtypes = [vp, vp, u32]
        _lib = lib
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None or a.size == 0 else a.ctypes.data


def _rel(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.int32)
    assert a.ndim == 2 and a.shape[1] == 2
    return a


def generate(spec, threads: int = 1) -> np.ndarray:
    """Host copy of a generated relation (same generator as the device).

    Zipf specs with s > 0 get their CDF table built here (ejo_zipf_cdf).
    threads > 1 generates row ranges in parallel (same rows)."""
    lib = load()
    out = np.empty((spec.n, 2), dtype=np.int32)
    keep = None
    if spec.kind == 2 and spec.zipf_s != 0.0 and not spec.cdf:
        keep = np.empty(spec.domain, dtype=np.float64)
        lib.ejo_zipf_cdf(spec.zipf_s, spec.domain, keep.ctypes.data)
        spec.cdf = keep.ctypes.data
    try:
        if spec.n and threads > 1:
            lib.ejo_generate_mt(C.byref(spec), out.ctypes.data, threads)
        elif spec.n:
            lib.ejo_generate(C.byref(spec), out.ctypes.data)
    finally:
        if keep is not None:
            spec.cdf = None
    return out


def join_digest(R, S, outer: bool = False, threads: int = 0, partitions: int = 1 << 20) -> tuple[int, int]:
    """(count, checksum) of the inner join (outer: the left outer join) of R
    and S without materialising its rows: the joins/multi_joins/hash
    restatement with every row fed to the order-independent checksum."""
    lib = load()
    R, S = _rel(R), _rel(S)
    nt = threads or os.cpu_count() or 8
    n, c = C.c_uint64(0), C.c_uint64(0)
    if lib.ejo_join_digest_mt(_p(R), len(R), _p(S), len(S), int(outer), partitions, nt, C.byref(n), C.byref(c)):
        raise MemoryError("ejo_join_digest_mt")
    return int(n.value), int(c.value)


def star_digest(F1, F2, D1, D2, threads: int = 0, nb_bucket: int = 1 << 20) -> tuple[int, int]:
    """(count, checksum) of the 3-way star join without materialising its rows."""
    lib = load()
    F1, F2, D1, D2 = (_rel(x) for x in (F1, F2, D1, D2))
    nt = threads or os.cpu_count() or 8
    n, c = C.c_uint64(0), C.c_uint64(0)
    if lib.ejo_star_digest_mt(_p(F1), _p(F2), len(F1), _p(D1), len(D1), _p(D2), len(D2), nb_bucket, nt,
                              C.byref(n), C.byref(c)):
        raise MemoryError("ejo_star_digest_mt")
    return int(n.value), int(c.value)


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


# ---- distance joins ------------------------------------------------------------
# TUPLE {int id; double val[dims]}; rows as the reference lays them out: dims 2
# {lid, lval[2], rid, rval[2]} (blockJoin_gpu/complex_block/dire_join/tuple.h:25-30),
# dims 3 {lval[3], rval[3], lid, rid} (CPU_JOIN/3d_cpu/nestLoopJoin.cc:28-33)
POINT_DTYPE = {d: np.dtype([("id", "<i4"), ("val", "<f8", (d,))], align=True) for d in (2, 3)}
POINT_RESULT_DTYPE = {
    2: np.dtype([("lid", "<i4"), ("lval", "<f8", (2,)), ("rid", "<i4"), ("rval", "<f8", (2,))], align=True),
    3: np.dtype([("lval", "<f8", (3,)), ("rval", "<f8", (3,)), ("lid", "<i4"), ("rid", "<i4")], align=True),
}
# the 2-D CPU program's row (joins/blockJoin_gpu/complex_block/2d_cpu/nestLoopJoin.cc:28-33)
REF_CPU_ROW2_DTYPE = np.dtype([("lval", "<f8", (2,)), ("rval", "<f8", (2,)), ("lid", "<i4"), ("rid", "<i4")])


def distance_join(dims: int, R, S, radius: float = 1.0, threads: int = 1) -> np.ndarray:
    """CPU_JOIN/3d_cpu (dims 3) / complex_block/2d_cpu (dims 2) restated: every
    (S, R) pair with sum_i (r.val[i] - l.val[i])^2 < radius^2, left-major order."""
    lib = load()
    R = np.ascontiguousarray(R, dtype=POINT_DTYPE[dims])
    S = np.ascontiguousarray(S, dtype=POINT_DTYPE[dims])
    n = int(lib.ejo_distance_join(dims, _p(R), len(R), _p(S), len(S), radius, None, 0, threads))
    if n == 2 ** 64 - 1:
        raise MemoryError("ejo_distance_join")
    out = np.zeros(max(n, 1), dtype=POINT_RESULT_DTYPE[dims])
    m = int(lib.ejo_distance_join(dims, _p(R), len(R), _p(S), len(S), radius, out.ctypes.data, n, threads))
    assert m == n
    return out[:n]


def point_rows_canon(rows: np.ndarray) -> np.ndarray:
    """Distance-join rows of any of the layouts as an int64 matrix
    [lid, rid, lval bits..., rval bits...] in lexicographic order: equal
    matrices mean the same rows, bit for bit."""
    rows = np.asarray(rows)
    d = rows.dtype["lval"].shape[0]
    m = np.empty((len(rows), 2 + 2 * d), dtype=np.int64)
    m[:, 0] = rows["lid"]
    m[:, 1] = rows["rid"]
    m[:, 2:2 + d] = np.ascontiguousarray(rows["lval"]).view(np.int64).reshape(-1, d)
    m[:, 2 + d:] = np.ascontiguousarray(rows["rval"]).view(np.int64).reshape(-1, d)
    if len(m):
        m = m[np.lexsort(m.T[::-1])]
    return m


def point_rows_digest(rows: np.ndarray) -> str:
    """sha256 of point_rows_canon(rows)."""
    import hashlib

    return hashlib.sha256(point_rows_canon(rows).tobytes()).hexdigest()
