"""ctypes binding of the engine's C ABI (include/ej.h).

The shared library is built in-tree by :mod:`eating_one_gb300.build`.  Loading
fails loudly when it is missing: there is no CPU fallback for any join.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

EJ_OK = 0
EJ_ERR_INVALID = 1
EJ_ERR_CAPACITY = 2
EJ_ERR_CUDA = 3
EJ_ERR_NOMEM = 4
EJ_ERR_TIMEOUT = 5
EJ_ERR_TOO_LARGE = 6
EJ_ERR_NO_DEVICE = 7
EJ_ERR_BUSY = 8
EJ_ERR_INTERNAL = 9
EJ_ERR_IO = 10

ALGO = {"hash": 0, "single_hash": 1, "bnl": 2, "hash_index": 3, "sort_index": 4, "left_outer": 5}

EJ_GEN_PERM, EJ_GEN_UNIFORM, EJ_GEN_ZIPF = 0, 1, 2


def _np():
    import numpy as np
    return np


def point_dtype(dims: int):
    """numpy dtype of ej_point2 / ej_point3: {int32 id; double val[dims]} (24 or 32 bytes)."""
    np = _np()
    if dims not in (2, 3):
        raise ValueError("dims must be 2 or 3")
    return np.dtype([("id", "<i4"), ("val", "<f8", (dims,))], align=True)


def point_result_dtype(dims: int):
    """numpy dtype of ej_point_result2 {lid, lval[2], rid, rval[2]} (48 bytes) or
    ej_point_result3 {lval[3], rval[3], lid, rid} (56 bytes)."""
    np = _np()
    if dims == 2:
        return np.dtype([("lid", "<i4"), ("lval", "<f8", (2,)), ("rid", "<i4"), ("rval", "<f8", (2,))], align=True)
    if dims == 3:
        return np.dtype([("lval", "<f8", (3,)), ("rval", "<f8", (3,)), ("lid", "<i4"), ("rid", "<i4")], align=True)
    raise ValueError("dims must be 2 or 3")


class GenSpec(C.Structure):
    """Mirror of ej_gen_spec (include/ej_gen.h)."""

    _fields_ = [
        ("kind", C.c_uint32),
        ("domain", C.c_uint32),
        ("seed", C.c_uint64),
        ("kseed", C.c_uint64),
        ("n", C.c_uint64),
        ("dup", C.c_uint32),
        ("absent_permille", C.c_uint32),
        ("val_base", C.c_int32),
        ("absent_base", C.c_int32),
        ("key_base", C.c_int32),
        ("reserved", C.c_uint32),
        ("zipf_s", C.c_double),
        ("cdf", C.c_void_p),
    ]


class JoinDesc(C.Structure):
    """Mirror of ej_join_desc (include/ej.h)."""

    _fields_ = [("R", C.c_void_p), ("nR", C.c_uint64), ("S", C.c_void_p), ("nS", C.c_uint64),
                ("out", C.c_void_p), ("out_cap", C.c_uint64)]


class ServerConfig(C.Structure):
    """Mirror of ej_server_config (include/ej.h)."""

    _fields_ = [("device", C.c_int), ("mode", C.c_int), ("lanes", C.c_uint32), ("max_batch_joins", C.c_uint32),
                ("lane_bytes", C.c_uint64), ("max_queued", C.c_uint32), ("flags", C.c_uint32)]


class Completion(C.Structure):
    """Mirror of ej_completion (include/ej.h)."""

    _fields_ = [("tag", C.c_uint64), ("count", C.c_uint64), ("status", C.c_int32), ("batch_joins", C.c_uint32),
                ("arrival_ns", C.c_uint64), ("launch_ns", C.c_uint64), ("done_ns", C.c_uint64),
                ("checksum", C.c_uint64)]


class ChunkConfig(C.Structure):
    _fields_ = [("r_block_rows", C.c_uint64), ("s_chunk_rows", C.c_uint64)]


class TuneEntry(C.Structure):
    """Mirror of ej_tune_entry (include/ej.h)."""

    _fields_ = [("log2_rows", C.c_uint32), ("partition_bits", C.c_int32), ("bucket_delta", C.c_int32),
                ("build", C.c_int32), ("table", C.c_int32), ("probe_warps", C.c_int32),
                ("reserved", C.c_int32 * 2)]


EJ_SERVE_BATCHED, EJ_SERVE_PER_JOIN = 0, 1
EJ_SERVE_CHECKSUM = 1
EJ_BUILD_PLANNER, EJ_BUILD_LSD, EJ_BUILD_MSD, EJ_BUILD_ONESWEEP = 0, 1, 2, 3
EJ_TABLE_FORMAT_PLANNER, EJ_TABLE_FORMAT_BUCKETS, EJ_TABLE_FORMAT_DIRECTORY = 0, 1, 2
EJ_TABLE_FILE_COUNTED, EJ_TABLE_FILE_RAW = 0, 1

_vp, _u64, _pu64, _i32 = C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64), C.c_int

# name -> argtypes (restype is ej_status = int unless listed in _RESTYPES)
_SIGS = {
    "ej_create": [C.c_int, C.POINTER(C.c_void_p)],
    "ej_destroy": [_vp],
    "ej_set_stream": [_vp, _vp],
    "ej_status_name": [_i32],
    "ej_last_error": [_vp],
    "ej_scratch_bytes": [_vp],
    "ej_trim": [_vp],
    "ej_set_timing": [_vp, _i32],
    "ej_last_phase_ms": [_vp, C.POINTER(C.c_float)],
    "ej_phase_totals": [_vp, C.POINTER(C.c_double), C.POINTER(C.c_uint32)],
    "ej_kernel_launches": [_vp],
    "ej_set_option": [_vp, _i32, C.c_int64],
    "ej_set_tuning": [_vp, _vp, C.c_uint32],
    "ej_hash_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_hash_join_count": [_vp, _vp, _u64, _vp, _u64, _pu64],
    "ej_hash_join_async": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _vp],
    "ej_sync_status": [_vp],
    "ej_single_hash_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_bnl_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_bnl_join_count": [_vp, _vp, _u64, _vp, _u64, _pu64],
    "ej_distance_join": [_vp, C.c_uint32, _vp, _u64, _vp, _u64, C.c_double, _vp, _u64, _pu64],
    "ej_distance_join_count": [_vp, C.c_uint32, _vp, _u64, _vp, _u64, C.c_double, _pu64],
    "ej_hash_index_build": [_vp, _vp, _u64, C.POINTER(C.c_void_p)],
    "ej_sort_index_build": [_vp, _vp, _u64, C.POINTER(C.c_void_p)],
    "ej_index_free": [_vp, _vp],
    "ej_index_join": [_vp, _vp, _vp, _u64, _vp, _u64, _pu64],
    "ej_index_join_count": [_vp, _vp, _vp, _u64, _pu64],
    "ej_index_merge_join": [_vp, _vp, _vp, _u64, _i32, _vp, _u64, _pu64],
    "ej_hash_index_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_sort_index_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_left_outer_join": [_vp, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_index_left_outer_join": [_vp, _vp, _vp, _u64, _vp, _u64, _pu64],
    "ej_star_join3": [_vp, _vp, _vp, _u64, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_join": [_vp, _i32, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_batch_hash_join": [_vp, _vp, C.c_uint32, _pu64],
    "ej_batch_hash_join_async": [_vp, _vp, C.c_uint32, _vp],
    "ej_server_create": [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)],
    "ej_server_submit": [_vp, C.POINTER(JoinDesc), _u64, _u64],
    "ej_server_poll": [_vp, C.POINTER(Completion), C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32],
    "ej_server_drain": [_vp],
    "ej_server_destroy": [_vp],
    "ej_now_ns": [],
    "ej_inject_alloc_failures": [C.c_uint32],
    "ej_join_host": [_vp, _i32, _vp, _u64, _vp, _u64, _vp, _u64, _pu64],
    "ej_join_host_chunked": [_vp, _i32, _vp, _u64, _vp, _u64, _vp, _u64, _pu64, _vp],
    "ej_exclusive_scan_u32": [_vp, _vp, _u64, _vp],
    "ej_exclusive_scan_u32_noalloc": [_vp, _u64, _vp, _vp],
    "ej_generate": [_vp, C.POINTER(GenSpec), _vp],
    "ej_checksum": [_vp, _vp, _u64, C.c_uint32, _pu64],
    "ej_table_file_rows": [C.c_char_p, _i32, _pu64],
    "ej_table_file_read": [C.c_char_p, _i32, _vp, _u64, _pu64],
    "ej_table_load": [_vp, C.c_char_p, _i32, _vp, _u64, _pu64],
    "ej_table_save": [_vp, C.c_char_p, _i32, _vp, _u64],
}
_RESTYPES = {"ej_status_name": C.c_char_p, "ej_last_error": C.c_char_p, "ej_scratch_bytes": C.c_uint64,
             "ej_kernel_launches": C.c_uint64, "ej_now_ns": C.c_uint64}
EJ_PHASES = 4  # build | partition | count | write

_lib = None


def exported_names() -> list[str]:
    return list(_SIGS)


def load(path: str | None = None) -> C.CDLL:
    """Load the engine library (building nothing); raises when it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "eating_one_gb300 CUDA library not built (%s missing); run eating_one_gb300.build.build()" % p)
    lib = C.CDLL(p)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    if path is None:
        _lib = lib
    return lib


def read_table_file(path: str, fmt: int = EJ_TABLE_FILE_COUNTED):
    """A table file read into host memory by the library (no GPU needed):
    an (n, 2) int32 numpy array of TUPLE{key, val} rows."""
    import numpy as np

    lib = load()
    n = C.c_uint64(0)
    st = lib.ej_table_file_rows(os.fsencode(path), fmt, C.byref(n))
    if st != EJ_OK:
        raise OSError("%s: %s" % (path, lib.ej_status_name(st).decode()))
    out = np.empty((n.value, 2), dtype=np.int32)
    st = lib.ej_table_file_read(os.fsencode(path), fmt, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n))
    if st != EJ_OK:
        raise OSError("%s: %s" % (path, lib.ej_status_name(st).decode()))
    return out
