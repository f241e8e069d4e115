"""Distance join on the GPU against the oracle: bit-exact rows (every double
compared by its bits, tolerance 0), and the reference's own recorded runs."""
import math

import numpy as np
import pytest

from eating_one_gb300 import native
from eating_one_gb300.engine import JoinError
from eating_one_gb300.workloads import distance_points, distance_workload
from oracle import oracle as O
from tests.golden import boundary_points, distance_cases

pytestmark = pytest.mark.gpu


def _gpu_rows(engine, dims, R, S, radius=1.0):
    rows = engine.distance_join(engine.points_to_device(R), engine.points_to_device(S), dims, radius)
    return engine.rows_to_numpy(rows, dims)


def _same(engine, dims, R, S, radius=1.0, threads=8):
    got = O.point_rows_canon(_gpu_rows(engine, dims, R, S, radius))
    want = O.point_rows_canon(O.distance_join(dims, R, S, radius, threads=threads))
    assert got.shape == want.shape, (got.shape, want.shape)
    assert np.array_equal(got, want)
    return len(want)


@pytest.mark.parametrize("case", distance_cases(), ids=lambda c: c["case"])
def test_reference_runs(engine, case):
    """Rows equal, bit for bit, to what the reference program produced."""
    rows = _gpu_rows(engine, case["dims"], case["R"], case["S"])
    assert len(rows) == case["count"]
    assert O.point_rows_digest(rows) == case["digest"]


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("radius", [1.0, 0.5, 2.5, -1.0, 0.0, 1e-300, 1e20, float("inf"), float("nan")])
def test_radius(engine, dims, radius):
    R, S = boundary_points(dims, 700, 900, 1000 + dims)
    n = _same(engine, dims, R, S, radius)
    if radius in (0.0, 1e-300) or radius != radius:
        assert n == 0
    if radius in (1e20, float("inf")):
        # every pair whose squared distance is finite (no NaN, no inf - inf, no overflow)
        assert n > 0.9 * len(R) * len(S)


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("nR,nS", [(1, 1), (1, 5000), (5000, 1), (4095, 4097), (4096 * 3 + 17, 4096 * 2 + 3),
                                   (20000, 700)])
def test_ragged_sizes(engine, dims, nR, nS):
    # a box sized so that every point has a few neighbours
    box = (max(nR, nS) * (4.2 if dims == 3 else 3.2)) ** (1.0 / dims) * 0.8
    R, S = boundary_points(dims, nR, nS, nR * 7 + nS, box=box)
    _same(engine, dims, R, S)


@pytest.mark.parametrize("dims", [2, 3])
def test_empty_sides(engine, dims):
    R, S = distance_points(dims, 100, 100, 3)
    for a, b in ((R[:0], S), (R, S[:0]), (R[:0], S[:0])):
        assert len(_gpu_rows(engine, dims, a, b)) == 0
        assert engine.distance_join_count(engine.points_to_device(a), engine.points_to_device(b), dims) == 0


@pytest.mark.parametrize("dims", [2, 3])
def test_reference_shaped(engine, dims):
    R, S = distance_points(dims, 1 << 14, 1 << 14, 77 + dims)
    assert _same(engine, dims, R, S) == math.ceil(0.1 * (1 << 14))


@pytest.mark.parametrize("dims", [2, 3])
def test_count_only(engine, dims):
    R, S = boundary_points(dims, 3000, 5000, 5 + dims, box=40.0)
    dR, dS = engine.points_to_device(R), engine.points_to_device(S)
    n = len(O.distance_join(dims, R, S, threads=8))
    assert engine.distance_join_count(dR, dS, dims) == n


def test_capacity(engine):
    R, S = boundary_points(3, 500, 600, 8)
    n = len(O.distance_join(3, R, S))
    import torch

    out = torch.empty((n - 1, 56), dtype=torch.uint8, device=engine.device)
    with pytest.raises(JoinError) as e:
        engine.distance_join(engine.points_to_device(R), engine.points_to_device(S), 3, 1.0, out=out)
    assert e.value.status == native.EJ_ERR_CAPACITY


def test_invalid_arguments(engine):
    import ctypes as C

    R, S = distance_points(3, 10, 10, 1)
    dR, dS = engine.points_to_device(R), engine.points_to_device(S)
    cnt = C.c_uint64(0)
    lib = engine.lib
    assert lib.ej_distance_join_count(engine.h, 4, dR.data_ptr(), 10, dS.data_ptr(), 10, 1.0,
                                      C.byref(cnt)) == native.EJ_ERR_INVALID
    assert lib.ej_distance_join_count(engine.h, 3, dR.data_ptr() + 4, 9, dS.data_ptr(), 10, 1.0,
                                      C.byref(cnt)) == native.EJ_ERR_INVALID
    assert lib.ej_distance_join_count(engine.h, 3, None, 10, dS.data_ptr(), 10, 1.0,
                                      C.byref(cnt)) == native.EJ_ERR_INVALID
    assert lib.ej_distance_join(engine.h, 3, dR.data_ptr(), 10, dS.data_ptr(), 10, 1.0, None, 5,
                                C.byref(cnt)) == native.EJ_ERR_INVALID


@pytest.mark.parametrize("name", ["d2", "d3"])
def test_full_size_copies(engine, name):
    """Full benchmark size (2^19 x 2^19 points): the matches are exactly the
    generator's copies (distinct integer values are at least 1 apart in every
    dimension), each row pairing a left point with the right point it copied."""
    dims, R, S = distance_workload(name)
    dR, dS = engine.points_to_device(R), engine.points_to_device(S)
    rows = engine.rows_to_numpy(engine.distance_join(dR, dS, dims), dims)
    assert len(rows) == math.ceil(0.1 * len(R)) == engine.distance_join_count(dR, dS, dims)
    assert len(np.unique(rows["lid"])) == len(rows)
    n_r = len(R)
    assert np.array_equal(rows["lval"], S["val"][rows["lid"] - n_r - 1])
    assert np.array_equal(rows["rval"], R["val"][rows["rid"] - 1])
    assert np.array_equal(rows["lval"], rows["rval"])
