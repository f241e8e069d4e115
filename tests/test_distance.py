"""Distance join: the oracle against the reference's own runs, and host-side logic (no GPU).

The reference programs joins/CPU_JOIN/3d_cpu and
joins/blockJoin_gpu/complex_block/2d_cpu were run on the inputs stored in
tests/golden/distance.npz (tests/golden/make_golden.py); their match count and
the sha256 of their canonical rows are the known answers here.
"""
import math

import numpy as np
import pytest

from eating_one_gb300 import native
from eating_one_gb300.workloads import distance_points
from oracle import oracle as O
from tests.golden import boundary_points, distance_cases

CASES = distance_cases()


def test_fixtures_present():
    assert {c["case"] for c in CASES} == {"ref_shape_2d", "ref_shape_3d", "boundary_2d", "boundary_3d"}


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["case"])
def test_oracle_pinned_to_reference(case):
    rows = O.distance_join(case["dims"], case["R"], case["S"])
    assert len(rows) == case["count"]
    assert O.point_rows_digest(rows) == case["digest"]


def _numpy_count(R, S, order, dtype=np.float64):
    with np.errstate(all="ignore"):
        r = R["val"].astype(dtype)
        l_ = S["val"].astype(dtype)
        t = r[None, :, :] - l_[:, None, :]
        sq = t * t
        temp = np.zeros(sq.shape[:2], dtype)
        dims = range(sq.shape[2]) if order == "forward" else reversed(range(sq.shape[2]))
        for i in dims:
            temp = temp + sq[:, :, i]
        return int((temp < 1.0).sum())


def test_boundary_fixtures_discriminate_rounding():
    """The boundary inputs separate the reference's evaluation from near misses:
    summing the squares in the other order, or in float32, changes the answer."""
    b3 = next(c for c in CASES if c["case"] == "boundary_3d")
    b2 = next(c for c in CASES if c["case"] == "boundary_2d")
    assert _numpy_count(b3["R"], b3["S"], "forward") == b3["count"]
    assert _numpy_count(b3["R"], b3["S"], "reverse") != b3["count"]
    assert _numpy_count(b3["R"], b3["S"], "forward", np.float32) != b3["count"]
    assert _numpy_count(b2["R"], b2["S"], "forward") == b2["count"]
    assert _numpy_count(b2["R"], b2["S"], "forward", np.float32) != b2["count"]


@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_threads_same_rows(dims):
    R, S = boundary_points(dims, 300, 500, 99)
    one = O.distance_join(dims, R, S, threads=1)
    four = O.distance_join(dims, R, S, threads=4)
    assert one.tobytes() == four.tobytes()


@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_radius(dims):
    R, S = boundary_points(dims, 200, 300, 5)
    base = O.point_rows_canon(O.distance_join(dims, R, S, 1.0))
    # radius enters as radius^2: the sign does not matter
    assert np.array_equal(O.point_rows_canon(O.distance_join(dims, R, S, -1.0)), base)
    assert len(O.distance_join(dims, R, S, 0.0)) == 0
    assert len(O.distance_join(dims, R, S, float("nan"))) == 0
    small, big = len(O.distance_join(dims, R, S, 0.5)), len(O.distance_join(dims, R, S, 2.0))
    assert small < len(base) < big


def test_oracle_empty():
    for dims in (2, 3):
        R, S = distance_points(dims, 10, 10, 1)
        assert len(O.distance_join(dims, R[:0], S)) == 0
        assert len(O.distance_join(dims, R, S[:0])) == 0


def test_dtypes_match_header_layouts():
    # include/ej.h: ej_point2 24, ej_point3 32, ej_point_result2 48, ej_point_result3 56 bytes
    assert [native.point_dtype(d).itemsize for d in (2, 3)] == [24, 32]
    assert [native.point_result_dtype(d).itemsize for d in (2, 3)] == [48, 56]
    for d in (2, 3):
        assert native.point_dtype(d) == O.POINT_DTYPE[d]
        assert native.point_result_dtype(d) == O.POINT_RESULT_DTYPE[d]
    r2 = native.point_result_dtype(2)
    assert [r2.fields[f][1] for f in ("lid", "lval", "rid", "rval")] == [0, 8, 24, 32]
    r3 = native.point_result_dtype(3)
    assert [r3.fields[f][1] for f in ("lval", "rval", "lid", "rid")] == [0, 24, 48, 52]


@pytest.mark.parametrize("n", [1000, 32768])
def test_generator_shape(n):
    """Reference-shaped points: unique integer values, ceil(0.1 |R|) left copies
    (the reference's 2-D log prints 3277 at 32768 x 32768)."""
    for dims in (2, 3):
        R, S = distance_points(dims, n, n, 17)
        assert (R["val"] == R["val"][:, :1]).all() and (S["val"] == S["val"][:, :1]).all()
        assert len(np.unique(R["val"][:, 0])) == n
        copies = len(np.intersect1d(R["val"][:, 0], S["val"][:, 0]))
        assert copies == math.ceil(0.1 * n)
    assert copies == (3277 if n == 32768 else 100)
