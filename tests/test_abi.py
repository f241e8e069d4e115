"""CPU tests of the C ABI boundary: the library builds, loads and exports every
entry point include/ej.h declares.  No compute call is made without a GPU."""
import ctypes as C
import os
import re

import pytest

from eating_one_gb300 import native
from eating_one_gb300.build import INCLUDE, build

HEADER = os.path.join(INCLUDE, "ej.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(ej_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build()
    return native.load()


def test_header_lists_entry_points():
    names = declared_functions()
    assert "ej_hash_join" in names and "ej_bnl_join" in names and "ej_star_join3" in names
    assert len(names) >= 30


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    assert set(declared_functions()) == set(native.exported_names())


def test_status_names(lib):
    assert lib.ej_status_name(native.EJ_ERR_CAPACITY) == b"EJ_ERR_CAPACITY"
    assert lib.ej_status_name(42) == b"EJ_ERR_UNKNOWN"


def test_null_arguments_rejected(lib):
    assert lib.ej_create(0, None) == native.EJ_ERR_INVALID
    assert lib.ej_destroy(None) == native.EJ_ERR_INVALID
    assert lib.ej_hash_join(None, None, 0, None, 0, None, 0, None) == native.EJ_ERR_INVALID
    assert lib.ej_last_error(None) == b""


def test_structs_match_reference_layout():
    from eating_one_gb300.native import GenSpec
    assert C.sizeof(GenSpec) == 72
    # TUPLE is 8 bytes and RESULT 16 (joins/hashJoin_gpu/main_street/tuple.h:43-53)
    text = open(HEADER).read()
    assert "typedef struct ej_tuple { int32_t key; int32_t val; } ej_tuple;" in text
    assert "typedef struct ej_result { int32_t rkey; int32_t rval; int32_t lkey; int32_t lval; } ej_result;" in text
