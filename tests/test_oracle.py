"""CPU tests: the oracle against the reference's own outputs and against brute force.

These pin the oracle before any GPU result is compared with it:
  - the reference's join_ori known-answer tables (four reference programs all
    print resultVal = sum of rval over all matches = 50438235);
  - counts and row checksums printed/materialised by the unmodified
    joins/CPU_JOIN programs on seeded relations (tests/golden/reference_runs.json,
    made by tests/golden/make_golden.py);
  - a numpy brute-force join on small random relations, negative keys included.
"""
import numpy as np
import pytest

from eating_one_gb300.workloads import workload
from oracle import oracle as O
from tests import golden

JOINS = {
    "hash": O.hash_join,
    "hash_index": O.hash_index_join,
    "sort_index": O.sort_index_join,
    "bnl": O.bnl_join,
}


def brute_force(R, S):
    rows = []
    by_val = {}
    for k, v in R:
        by_val.setdefault(int(v), []).append(int(k))
    for k, v in S:
        for rk in by_val.get(int(v), []):
            rows.append((rk, int(v), int(k), int(v)))
    return np.array(rows, dtype=np.int32).reshape(-1, 4)


@pytest.mark.parametrize("name", list(JOINS))
def test_join_ori_known_answer(name):
    R, S = golden.join_ori()
    runs = golden.reference_runs()["join_ori"]
    rows = JOINS[name](R, S)
    assert len(rows) == 1002230
    # every reference program prints the same sum of rval (int arithmetic, no overflow here)
    assert set(runs.values()) == {int(rows[:, 1].astype(np.int64).sum())} == {50438235}
    assert np.all(rows[:, 1] == rows[:, 3])


@pytest.mark.parametrize("case", range(len(golden.reference_runs()["cpu_join"])))
def test_against_reference_programs(case):
    run = golden.reference_runs()["cpu_join"][case]
    w = workload(run["workload"], run["scale"])
    w["R"].key_base = 1
    w["S"].key_base = 1 + w["R"].n
    R, S = O.generate(w["R"]), O.generate(w["S"])
    assert (len(R), len(S)) == (run["nR"], run["nS"])
    fn = {"hash_cpu": O.hash_join, "inner_cpu": O.hash_index_join,
          "sortindex_cpu": O.sort_index_join, "block_cpu": O.bnl_join}[run["program"]]
    rows = fn(R, S)
    assert len(rows) == run["count"]
    if run["checksum"] is not None:
        assert O.checksum(rows) == int(run["checksum"])


@pytest.mark.parametrize("seed", range(4))
def test_oracle_joins_match_brute_force(seed):
    rng = np.random.default_rng(seed)
    lo, hi = [(0, 50), (-30, 30), (-(2 ** 31), 2 ** 31 - 1), (0, 3)][seed]
    R = np.stack([np.arange(300), rng.integers(lo, hi, 300)], axis=1).astype(np.int32)
    S = np.stack([np.arange(1000, 2700), rng.integers(lo, hi, 1700)], axis=1).astype(np.int32)
    ref = O.canon(brute_force(R, S))
    for name, fn in JOINS.items():
        assert np.array_equal(O.canon(fn(R, S)), ref), name
    assert O.hash_join_count(R, S) == len(ref)


def test_left_outer_semantics():
    rng = np.random.default_rng(5)
    R = np.stack([np.arange(200), rng.integers(0, 100, 200)], axis=1).astype(np.int32)
    S = np.stack([np.arange(500), rng.integers(0, 200, 500)], axis=1).astype(np.int32)
    out = O.left_outer_join(R, S)
    inner = O.hash_index_join(R, S)
    unmatched = ~np.isin(S[:, 1], R[:, 1])
    null_rows = out[out[:, 0] == -(2 ** 31)]
    assert len(out) == len(inner) + unmatched.sum()
    assert np.array_equal(np.sort(null_rows[:, 2]), np.sort(S[unmatched, 0]))
    assert np.all(null_rows[:, 1] == -(2 ** 31))


def test_star_semantics():
    rng = np.random.default_rng(6)
    F1 = np.stack([np.arange(400), rng.integers(0, 30, 400)], axis=1).astype(np.int32)
    F2 = np.stack([np.arange(400), rng.integers(0, 20, 400)], axis=1).astype(np.int32)
    D1 = np.stack([np.arange(50), rng.integers(0, 40, 50)], axis=1).astype(np.int32)
    D2 = np.stack([np.arange(30), rng.integers(0, 25, 30)], axis=1).astype(np.int32)
    out = O.star_join3(F1, F2, D1, D2)
    expect = []
    for f in range(400):
        for d1 in D1[D1[:, 1] == F1[f, 1]]:
            for d2 in D2[D2[:, 1] == F2[f, 1]]:
                expect.append([d1[0], d1[1], F1[f, 0], F1[f, 1], d2[0], d2[1], F2[f, 0], F2[f, 1]])
    assert np.array_equal(O.canon(out), O.canon(np.array(expect, dtype=np.int32).reshape(-1, 8)))


def test_generators():
    w = workload("c3_s1.0", scale=8)
    R, S = O.generate(w["R"]), O.generate(w["S"])
    vals, counts = np.unique(R[:, 1], return_counts=True)
    assert len(vals) == 1 << 16 and np.all(counts == 4)  # 2^16 distinct keys, each x4
    assert np.array_equal(np.sort(vals), np.sort(np.unique(vals)))
    absent = S[:, 1] >= 1 << 30
    assert abs(absent.mean() - 0.1) < 0.01
    # Zipf s=1: the most frequent present key is about 1/H(n) of the present rows
    present = S[~absent, 1]
    top = np.unique(present, return_counts=True)[1].max() / len(present)
    h = np.sum(1.0 / np.arange(1, (1 << 16) + 1))
    assert abs(top - 1.0 / h) < 0.01
    c1 = workload("c1", scale=4)
    R1 = O.generate(c1["R"])
    assert np.array_equal(np.sort(R1[:, 1]), np.arange(1 << 16))  # a permutation
    assert np.array_equal(R1[:, 0], np.arange(1 << 16))


def test_checksum_order_independent():
    rng = np.random.default_rng(1)
    rows = rng.integers(-(2 ** 31), 2 ** 31 - 1, size=(1000, 4)).astype(np.int32)
    assert O.checksum(rows) == O.checksum(rows[::-1].copy())
    rows2 = rows.copy()
    rows2[5, 2] ^= 1
    assert O.checksum(rows) != O.checksum(rows2)


@pytest.mark.parametrize("threads,partitions", [(1, 1 << 17), (4, 1 << 10), (7, 3)])
def test_multithreaded_restatement(threads, partitions):
    """joins/multi_joins/hash restated with pthreads: the same multiset as the
    single-threaded hash_cpu restatement, and the join_ori known answer."""
    rng = np.random.default_rng(threads)
    for nR, nS, lo, hi in ((0, 10, 0, 5), (10, 0, 0, 5), (1000, 5000, -2 ** 31, 2 ** 31 - 1),
                           (3, 100000, 0, 4), (12345, 54321, -1000, 1000)):
        R = np.stack([np.arange(nR), rng.integers(lo, hi, nR)], 1).astype(np.int32).reshape(-1, 2)
        S = np.stack([np.arange(nS), rng.integers(lo, hi, nS)], 1).astype(np.int32).reshape(-1, 2)
        got = O.hash_join_mt(R, S, threads=threads, partitions=partitions)
        assert np.array_equal(O.canon(got), O.canon(O.hash_join(R, S)))
    R, S = golden.join_ori()
    rows = O.hash_join_mt(R, S, threads=threads, partitions=partitions)
    assert len(rows) == 1002230 and int(rows[:, 1].astype(np.int64).sum()) == 50438235


@pytest.mark.parametrize("name", ["c3_s0.0", "c3_s1.0", "c4"])
def test_digest_matches_materialised_join(name):
    """The full-size goldens come from ejo_join_digest_mt: at a small size its
    count and checksum equal those of the materialised single-threaded joins,
    inner and left outer, for any thread and partition count."""
    w = workload(name, 8)
    R, S = O.generate(w["R"]), O.generate(w["S"], threads=3)
    assert np.array_equal(S, O.generate(w["S"]))
    inner, outer = O.hash_join(R, S), O.left_outer_join(R, S)
    for threads, parts in ((1, 1 << 20), (3, 1 << 14), (8, 4099)):
        assert O.join_digest(R, S, threads=threads, partitions=parts) == (len(inner), O.checksum(inner))
        assert O.join_digest(R, S, outer=True, threads=threads, partitions=parts) == (len(outer), O.checksum(outer))


def test_star_digest_matches_materialised_join():
    w = workload("c4_star", 7)
    t = {k: O.generate(v) for k, v in w.items()}
    rows = O.star_join3(t["F1"], t["F2"], t["D1"], t["D2"])
    for threads in (1, 5):
        assert O.star_digest(t["F1"], t["F2"], t["D1"], t["D2"], threads=threads) == (len(rows), O.checksum(rows))


def test_fullsize_goldens_cover_the_bench_workloads():
    g = golden.fullsize()
    for name in ("c3_s0.0", "c3_s0.75", "c3_s1.0"):
        assert g[name]["R"] == 1 << 26 and g[name]["S"] == 1 << 28
        assert 9.6e8 < g[name]["inner"]["count"] < 9.7e8
    assert g["c4"]["outer"]["count"] == 1 << 26
    assert g["c4_star"]["star"]["count"] == 1 << 26


@pytest.mark.parametrize("threads", [1, 2, 5])
def test_multithreaded_join_any_thread_count(threads):
    rng = np.random.default_rng(threads)
    R = np.stack([np.arange(3000), rng.integers(0, 500, 3000)], axis=1).astype(np.int32)
    S = np.stack([np.arange(9000), rng.integers(-20, 520, 9000)], axis=1).astype(np.int32)
    assert np.array_equal(O.canon(O.hash_join_mt(R, S, threads=threads, partitions=97)), O.canon(O.hash_join(R, S)))
