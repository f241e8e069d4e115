"""Seeded synthetic join workloads (generator specs, see include/ej_gen.h).

The reference draws unique values from [0, SELECTIVITY) with time-seeded
rand() (joins/hashJoin_gpu/main_street/hj.cc:62-160); the benchmark
configurations below instead fix the relation sizes and key distributions and
a seed per configuration (0xE1A00000 + configuration number):

  c1       hash join, R 2^20 unique keys (a permutation of [0, 2^20)),
           S 2^22 keys uniform in [0, 2^20): exactly |S| results
  c2       block nested-loop join, R 2^16 and S 2^20 keys uniform in
           [0, 2^16) on both sides (many-to-many)
  c3_sX    skewed hash join, R 2^26 = 2^24 distinct keys x 4 (shuffled),
           S 2^28 keys: 10% from the absent range [2^30, 2^30 + 2^24),
           else Zipf(s = X) ranks over R's 2^24 keys, X in {0, 0.75, 1}
  c4       index / outer joins, R 2^24 unique keys, S 2^26 keys: half uniform
           over R's keys, half from the absent range
  c4_star  star join, F 2^26 rows with two foreign keys uniform over the 2^20
           unique keys of D1 and D2

`scale=k` divides every size and key domain by 2^k (same shapes, smaller).
Row ids (.key) number each relation from 0.
"""
from __future__ import annotations

from .native import EJ_GEN_PERM, EJ_GEN_UNIFORM, EJ_GEN_ZIPF, GenSpec

SEED_BASE = 0xE1A00000
ABSENT_BASE = 1 << 30


def make_spec(kind: int, n: int, domain: int, seed: int, kseed: int = 0, dup: int = 1,
              absent_permille: int = 0, val_base: int = 0, absent_base: int = ABSENT_BASE,
              key_base: int = 0, zipf_s: float = 0.0) -> GenSpec:
    s = GenSpec()
    s.kind, s.n, s.domain, s.seed, s.kseed = kind, n, domain, seed, kseed
    s.dup, s.absent_permille, s.val_base, s.absent_base, s.key_base = dup, absent_permille, val_base, absent_base, key_base
    s.zipf_s, s.cdf, s.reserved = zipf_s, None, 0
    return s


def _seeds(config: int):
    base = SEED_BASE + config
    return base * 16 + 1, base * 16 + 2, base * 16 + 3, base * 16 + 4


def workload(name: str, scale: int = 0) -> dict[str, GenSpec]:
    """Generator specs of a named workload: keys 'R', 'S' (or 'F1', 'F2', 'D1', 'D2')."""
    sh = scale
    if name == "c1":
        rs, ss, ks, _ = _seeds(1)
        d = 1 << (20 - sh)
        return {"R": make_spec(EJ_GEN_PERM, d, d, rs, ks),
                "S": make_spec(EJ_GEN_UNIFORM, 1 << (22 - sh), d, ss)}
    if name == "c2":
        rs, ss, _, _ = _seeds(2)
        d = 1 << (16 - sh)
        return {"R": make_spec(EJ_GEN_UNIFORM, 1 << (16 - sh), d, rs),
                "S": make_spec(EJ_GEN_UNIFORM, 1 << (20 - sh), d, ss)}
    if name.startswith("c3_s"):
        s = float(name[4:])
        rs, ss, ks, _ = _seeds(3)
        d = 1 << (24 - sh)
        return {"R": make_spec(EJ_GEN_PERM, 4 * d, d, rs, ks, dup=4),
                "S": make_spec(EJ_GEN_ZIPF, 1 << (28 - sh), d, ss + int(s * 100), ks, absent_permille=100,
                               zipf_s=s)}
    if name == "c4":
        rs, ss, ks, _ = _seeds(4)
        d = 1 << (24 - sh)
        return {"R": make_spec(EJ_GEN_PERM, d, d, rs, ks),
                "S": make_spec(EJ_GEN_ZIPF, 1 << (26 - sh), d, ss, ks, absent_permille=500)}
    if name == "c4_star":
        rs, ss, ks, k2 = _seeds(5)
        d = 1 << (20 - sh)
        nf = 1 << (26 - sh)
        return {"D1": make_spec(EJ_GEN_PERM, d, d, rs, ks),
                "D2": make_spec(EJ_GEN_PERM, d, d, rs + 7, k2),
                "F1": make_spec(EJ_GEN_ZIPF, nf, d, ss, ks),
                "F2": make_spec(EJ_GEN_ZIPF, nf, d, ss + 7, k2)}
    raise KeyError(name)


# distance joins: the reference's logged 2-D runs go up to 2^19 x 2^19 points
# (joins/blockJoin_gpu/complex_block/2d_cpu/nohup.out)
DIST_WORKLOADS = {"d2": (2, 19), "d3": (3, 19)}


def distance_workload(name: str, scale: int = 0, seed: int | None = None):
    """(dims, R, S) of a named distance workload: |R| = |S| = 2^(log2 - scale)."""
    dims, lg = DIST_WORKLOADS[name]
    n = 1 << (lg - scale)
    return (dims,) + distance_points(dims, n, n, SEED_BASE + 16 + dims if seed is None else seed)


def distance_points(dims: int, n_right: int, n_left: int, seed: int, match_rate: float = 0.1,
                    selectivity: int = 1000000000):
    """Seeded points shaped as the reference's distance-join generator
    (joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc:114-186): every point has one
    integer value in [0, selectivity) in all dimensions, unique over both
    relations, except that every l_diff-th left point (l_diff = n_left /
    (match_rate n_right)) copies the values of a distinct random right point
    until ceil(match_rate n_right) have been copied.  Ids count from 1, right
    points first.  Returns (R, S) as numpy arrays of native.point_dtype(dims)."""
    import math

    import numpy as np

    from .native import point_dtype

    rng = np.random.Generator(np.random.PCG64(seed))
    need = n_right + n_left
    vals = np.empty(0, dtype=np.int64)
    while len(vals) < need:
        draw = np.unique(np.concatenate([vals, rng.integers(0, selectivity, size=need + need // 16 + 64)]))
        vals = draw
    vals = rng.permutation(vals)[:need].astype(np.float64)
    R = np.zeros(n_right, dtype=point_dtype(dims))
    S = np.zeros(n_left, dtype=point_dtype(dims))
    R["id"] = np.arange(1, n_right + 1, dtype=np.int32)
    S["id"] = np.arange(n_right + 1, n_right + n_left + 1, dtype=np.int32)
    rv = vals[:n_right]
    lv = vals[n_right:].copy()
    if match_rate > 0 and n_right and n_left:
        l_diff = max(1, int(n_left / (match_rate * n_right)))
        pos = np.arange(0, n_left, l_diff)[: math.ceil(match_rate * n_right)]
        pos = pos[: n_right]
        lv[pos] = rv[rng.choice(n_right, size=len(pos), replace=False)]
    R["val"] = rv[:, None]
    S["val"] = lv[:, None]
    return R, S


def alg_bytes(name: str, n_r: int, n_s: int, n_out: int) -> int:
    """Algorithmic bytes of one join (roofline numerator).

    Hash and outer joins: read both inputs once (8 B/tuple), one canonical
    partition pass reading and writing every tuple (16 B), write every 16-B
    result: 24(|R|+|S|) + 16|out|.  Index joins: 16|R| + 8|S| + 16|out|.
    """
    if name in ("hash_index", "sort_index", "index"):
        return 16 * n_r + 8 * n_s + 16 * n_out
    return 24 * (n_r + n_s) + 16 * n_out
