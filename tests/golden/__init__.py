"""Golden fixtures: loaders for the reference's join_ori tables and recorded reference runs."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def join_ori():
    """The reference's known-answer tables joins/join_ori/R and S as (n, 2) int32 arrays."""
    z = np.load(os.path.join(HERE, "join_ori.npz"))
    out = []
    for v in (z["R_val"], z["S_val"]):
        t = np.empty((len(v), 2), dtype=np.int32)
        t[:, 0] = np.arange(len(v))
        t[:, 1] = v
        out.append(t)
    return out[0], out[1]


def reference_runs():
    with open(os.path.join(HERE, "reference_runs.json")) as f:
        return json.load(f)


# ---- distance joins -------------------------------------------------------------
def point_dtype(dims):
    return np.dtype([("id", "<i4"), ("val", "<f8", (dims,))], align=True)


# offsets of length 1 (up to rounding): the pairs they plant sit on the
# reference's DISTANCE = 1 boundary, where the order of rounding decides
_UNIT_OFFSETS = {
    2: [(1.0, 0.0), (0.0, -1.0), (0.6, 0.8), (-0.8, 0.6), (0.28, -0.96), (0.5 ** 0.5, 0.5 ** 0.5),
        (0.96, 0.28), (-0.6, -0.8)],
    3: [(1.0, 0.0, 0.0), (0.0, 0.0, -1.0), (1 / 3, 2 / 3, 2 / 3), (2 / 7, -3 / 7, 6 / 7), (0.6, 0.8, 0.0),
        (-0.48, 0.6, 0.64), (3 ** -0.5, 3 ** -0.5, -(3 ** -0.5)), (0.0, -0.28, 0.96)],
}

# values whose single-precision screen takes a special path; each pairs with itself
_SPECIALS = [float("nan"), float("inf"), -float("inf"), -0.0, 0.0, 1e300, -1e300, 5e-324, 2.2e-308,
             3.4028234663852886e38, 3.5e38, -3.5e38, 1e9 + 0.5, 1e9 + 0.25, 16777217.0, -16777216.5]


def boundary_points(dims, n_right, n_left, seed, box=None):
    """Seeded points built to test the distance predicate at its edges:
    uniform points in [-box/2, box/2)^dims (negative values included); a third
    of S planted at a unit offset from an R point, each component nudged by
    -2..2 ulps; exact duplicates of R points; the _SPECIALS values (NaN, +-inf,
    +-0, subnormals, beyond float range, large magnitudes) in dimension 0 and in
    the last dimension of a few points on both sides, some in matching pairs.
    Ids count from 1, right points first.  Returns (R, S)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    box = box or (8.0 if dims == 3 else 16.0)
    R = np.zeros(n_right, dtype=point_dtype(dims))
    S = np.zeros(n_left, dtype=point_dtype(dims))
    R["id"] = np.arange(1, n_right + 1, dtype=np.int32)
    S["id"] = np.arange(n_right + 1, n_right + n_left + 1, dtype=np.int32)
    rv = rng.random((n_right, dims)) * box - box / 2
    sv = rng.random((n_left, dims)) * box - box / 2
    offs = np.array(_UNIT_OFFSETS[dims])
    k = n_left // 3
    src = rng.integers(0, n_right, k)
    o = offs[rng.integers(0, len(offs), k)]
    o = o + rng.integers(-2, 3, o.shape) * np.spacing(o)
    sv[:k] = rv[src] + o
    dup = n_left // 20
    sv[k:k + dup] = rv[rng.integers(0, n_right, dup)]
    # specials: R rows 0..m-1 and S rows k+dup..k+dup+2m-1
    m = len(_SPECIALS)
    if n_right >= m and n_left >= k + dup + 2 * m:
        sp = np.array(_SPECIALS)
        rv[:m, 0] = sp
        base = k + dup
        sv[base:base + m] = rv[:m]                       # same point: t = 0 unless NaN/inf
        sv[base:base + m, -1] += 0.5                     # then half a unit off in the last dimension
        sv[base + m:base + 2 * m, 0] = sp[::-1]
        sv[base + m:base + 2 * m, -1] = sp
    R["val"] = rv
    S["val"] = sv
    return R, S


def distance_cases():
    """The recorded reference runs of the distance programs, with their inputs:
    a list of dicts {case, dims, R, S, count, digest} (radius 1)."""
    runs = reference_runs().get("distance", [])
    z = np.load(os.path.join(HERE, "distance.npz"))
    out = []
    for r in runs:
        d = dict(r)
        d["R"] = z[r["case"] + "_R"].view(point_dtype(r["dims"])).reshape(-1)
        d["S"] = z[r["case"] + "_S"].view(point_dtype(r["dims"])).reshape(-1)
        out.append(d)
    return out


def fullsize():
    """The oracle's (count, checksum) of every full-size workload (tests/golden/make_fullsize.py)."""
    with open(os.path.join(HERE, "fullsize.json")) as f:
        return json.load(f)
