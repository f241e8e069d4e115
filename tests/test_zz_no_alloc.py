"""The scan entry point that allocates nothing, checked against the regular one.

ej_exclusive_scan_u32_noalloc serves callers that cannot allocate device
memory (their framework already owns the GPU's memory, they must avoid the
device-wide synchronisation of cudaMalloc/cudaFree, or they cannot keep an
ej_handle).  Its scratch is a static device array.  This file runs last so a
failure here leaves every other test already run; it passes alone in a fresh
process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from eating_one_gb300 import native

pytestmark = pytest.mark.gpu


def _scan_noalloc(lib, x: torch.Tensor) -> tuple[int, torch.Tensor]:
    out = torch.full((x.numel() + 1,), -1, dtype=torch.int64, device="cuda")
    st = lib.ej_exclusive_scan_u32_noalloc(C.c_void_p(x.data_ptr() if x.numel() else None), x.numel(),
                                           C.c_void_p(out.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, out


def test_noalloc_scan_matches_regular_scan(engine):
    lib = native.load()
    rng = np.random.default_rng(2024)
    # two calls in a row (the second reuses the scratch the first left behind),
    # the second smaller, so stale status words would show up as wrong prefixes
    for n in (3_000_001, 70_000):
        x = torch.from_numpy(rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32).view(np.int32)).cuda()
        st, got = _scan_noalloc(lib, x)
        assert st == native.EJ_OK
        ref = engine.exclusive_scan_u32(x)  # the existing entry point (handle scratch)
        assert torch.equal(got, ref)


def test_noalloc_scan_rejects_oversize_and_empty(engine):
    lib = native.load()
    x = torch.zeros(4, dtype=torch.int32, device="cuda")
    out = torch.zeros(5, dtype=torch.int64, device="cuda")
    st = lib.ej_exclusive_scan_u32_noalloc(C.c_void_p(x.data_ptr()), (1 << 28) + 1, C.c_void_p(out.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == native.EJ_ERR_TOO_LARGE
    st, got = _scan_noalloc(lib, torch.zeros(0, dtype=torch.int32, device="cuda"))
    assert st == native.EJ_OK and got.tolist() == [0]
