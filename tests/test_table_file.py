"""The reference's on-disk relation formats, read by the library on the host
(no GPU): EJ_TABLE_FILE_COUNTED (int32 n, then n TUPLEs, as
joins/hashJoin_gpu/main_street/TableBuild.cpp:113-140 writes them) and
EJ_TABLE_FILE_RAW (TUPLEs only, as the joins/join_ori R and S files)."""
import numpy as np
import pytest

from eating_one_gb300 import native
from tests import golden


def write_counted(path, rows, n=None):
    with open(path, "wb") as f:
        np.array([len(rows) if n is None else n], dtype=np.int32).tofile(f)
        np.ascontiguousarray(rows, dtype=np.int32).tofile(f)


def test_counted_and_raw_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    rows = rng.integers(-2 ** 31, 2 ** 31, size=(12345, 2), dtype=np.int64).astype(np.int32)
    write_counted(tmp_path / "t.tbl", rows)
    rows.tofile(tmp_path / "t.raw")
    assert np.array_equal(native.read_table_file(str(tmp_path / "t.tbl"), native.EJ_TABLE_FILE_COUNTED), rows)
    assert np.array_equal(native.read_table_file(str(tmp_path / "t.raw"), native.EJ_TABLE_FILE_RAW), rows)


def test_join_ori_files(tmp_path):
    R, S = golden.join_ori()
    R.tofile(tmp_path / "R")
    S.tofile(tmp_path / "S")
    assert np.array_equal(native.read_table_file(str(tmp_path / "R"), native.EJ_TABLE_FILE_RAW), R)
    got = native.read_table_file(str(tmp_path / "S"), native.EJ_TABLE_FILE_RAW)
    assert got.shape == (100000, 2) and np.array_equal(got, S)


def test_empty_tables(tmp_path):
    write_counted(tmp_path / "e.tbl", np.empty((0, 2), np.int32))
    open(tmp_path / "e.raw", "wb").close()
    assert native.read_table_file(str(tmp_path / "e.tbl")).shape == (0, 2)
    assert native.read_table_file(str(tmp_path / "e.raw"), native.EJ_TABLE_FILE_RAW).shape == (0, 2)


def test_malformed_files(tmp_path):
    rows = np.arange(20, dtype=np.int32).reshape(10, 2)
    write_counted(tmp_path / "short.tbl", rows[:5], n=10)  # header announces more rows than the file holds
    write_counted(tmp_path / "neg.tbl", rows, n=-1)
    with open(tmp_path / "odd.raw", "wb") as f:
        f.write(b"\0" * 12)  # not a whole number of tuples
    for name, fmt in (("short.tbl", native.EJ_TABLE_FILE_COUNTED), ("neg.tbl", native.EJ_TABLE_FILE_COUNTED),
                      ("odd.raw", native.EJ_TABLE_FILE_RAW), ("missing.tbl", native.EJ_TABLE_FILE_COUNTED)):
        with pytest.raises(OSError, match="EJ_ERR_IO"):
            native.read_table_file(str(tmp_path / name), fmt)


def test_capacity(tmp_path):
    import ctypes as C

    rows = np.arange(20, dtype=np.int32).reshape(10, 2)
    write_counted(tmp_path / "t.tbl", rows)
    lib = native.load()
    out = np.empty((4, 2), dtype=np.int32)
    n = C.c_uint64(0)
    st = lib.ej_table_file_read(str(tmp_path / "t.tbl").encode(), native.EJ_TABLE_FILE_COUNTED,
                                out.ctypes.data_as(C.c_void_p), 4, C.byref(n))
    assert st == native.EJ_ERR_CAPACITY and n.value == 10
