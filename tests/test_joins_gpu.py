"""Parity of every join entry point against the CPU oracle (exact result multisets).

Each test runs the CUDA path through the C ABI (libeating_one.so via ctypes)
and compares its rows, after canonical sorting, with the oracle's restatement
of the reference algorithm on the same seeded inputs.  Integer joins must be
bit-exact: there is no tolerance anywhere in this file.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from eating_one_gb300 import native
from eating_one_gb300.engine import JoinError
from eating_one_gb300.workloads import make_spec, workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INT_MIN, INT_MAX = -(2 ** 31), 2 ** 31 - 1


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


def same_multiset(gpu_rows: torch.Tensor, ref_rows: np.ndarray) -> None:
    g = O.canon(gpu_rows.cpu().numpy())
    r = O.canon(ref_rows)
    assert g.shape == r.shape, (g.shape, r.shape)
    assert np.array_equal(g, r)


def rel(rng, n, lo, hi, key_base=0):
    a = np.empty((n, 2), dtype=np.int32)
    a[:, 0] = np.arange(key_base, key_base + n, dtype=np.int64).astype(np.int32)
    a[:, 1] = rng.integers(lo, hi, size=n, dtype=np.int64).astype(np.int32)
    return a


ORACLE = {
    "hash": O.hash_join,
    "single_hash": O.hash_join,
    "hash_index": O.hash_index_join,
    "sort_index": O.sort_index_join,
    "bnl": O.bnl_join,
    "left_outer": O.left_outer_join,
}

CASES = [  # (nR, nS, key range) - unique-ish, many-to-many, heavy duplicates, ragged sizes
    (1000, 5000, (0, 1 << 20)),
    (4097, 8191, (0, 512)),
    (3, 100000, (0, 4)),
    (65536, 65536, (INT_MIN, INT_MAX)),
    (12345, 54321, (-1000, 1000)),
    (1, 1, (7, 8)),
    (2000, 3000, (0, 8)),  # ~250 rows per probe: groups larger than the write buffer
    (131072, 20, (5, 8)),  # three keys: long runs of empty buckets in the hash table
]


@pytest.mark.parametrize("algo", list(ORACLE))
@pytest.mark.parametrize("case", range(len(CASES)))
def test_small_parity(engine, algo, case):
    nR, nS, (lo, hi) = CASES[case]
    rng = np.random.default_rng(1000 + case)
    R, S = rel(rng, nR, lo, hi), rel(rng, nS, lo, hi, key_base=nR)
    got = engine.join(algo, dev(R), dev(S))
    same_multiset(got, ORACLE[algo](R, S))


@pytest.mark.parametrize("algo", list(ORACLE))
def test_empty_relations(engine, algo):
    rng = np.random.default_rng(7)
    R = rel(rng, 100, 0, 10)
    empty = np.zeros((0, 2), dtype=np.int32)
    for a, b in ((empty, R), (R, empty), (empty, empty)):
        got = engine.join(algo, dev(a), dev(b))
        assert got.shape[0] == len(ORACLE[algo](a, b))


def test_extreme_keys(engine):
    vals = np.array([INT_MIN, INT_MIN + 1, -1, 0, 1, INT_MAX - 1, INT_MAX], dtype=np.int32)
    R = np.stack([np.arange(len(vals) * 3, dtype=np.int32), np.repeat(vals, 3)], axis=1)
    S = np.stack([np.arange(100, 100 + len(vals) * 2, dtype=np.int32), np.tile(vals, 2)], axis=1)
    for algo in ORACLE:
        same_multiset(engine.join(algo, dev(R), dev(S)), ORACLE[algo](R, S))


@pytest.mark.parametrize("pb", [1, 3, 6, 7, 8])
def test_partitioned_probe(engine, pb):
    """Force the S radix-partition pass (taken automatically only for tables beyond L2)."""
    rng = np.random.default_rng(pb)
    R, S = rel(rng, 50000, 0, 30000), rel(rng, 200003, 0, 40000, key_base=50000)
    engine.set_option("partition_bits", pb)
    try:
        got_hash = engine.join("hash", dev(R), dev(S))
        got_outer = engine.join("left_outer", dev(R), dev(S))
    finally:
        engine.set_option("partition_bits", -1)
    same_multiset(got_hash, O.hash_join(R, S))
    same_multiset(got_outer, O.left_outer_join(R, S))


@pytest.mark.parametrize("pb", [5, 7])
def test_partitioned_probe_skewed(engine, pb):
    """One partition holds 90% of S: its (partition, group) segments span many warp tiles."""
    rng = np.random.default_rng(100 + pb)
    R = rel(rng, 40000, 0, 20000)
    S = rel(rng, 150001, 0, 25000, key_base=40000)
    S[rng.random(len(S)) < 0.9, 1] = R[7, 1]
    engine.set_option("partition_bits", pb)
    try:
        got_hash = engine.join("hash", dev(R), dev(S))
        got_outer = engine.join("left_outer", dev(R), dev(S))
    finally:
        engine.set_option("partition_bits", -1)
    same_multiset(got_hash, O.hash_join(R, S))
    same_multiset(got_outer, O.left_outer_join(R, S))


@pytest.mark.parametrize("delta", [-3, 3])
def test_bucket_sizes(engine, delta):
    rng = np.random.default_rng(11)
    R, S = rel(rng, 30000, 0, 5000), rel(rng, 70000, 0, 6000, key_base=30000)
    engine.set_option("bucket_bits_delta", delta)
    try:
        got = engine.join("hash", dev(R), dev(S))
    finally:
        engine.set_option("bucket_bits_delta", 0)
    same_multiset(got, O.hash_join(R, S))


def test_c1_full_size(engine):
    """Configuration C1 at full size: 2^20 unique R keys, 2^22 uniform S keys."""
    w = workload("c1")
    R, S = O.generate(w["R"]), O.generate(w["S"])
    Rd, Sd = engine.generate(w["R"]), engine.generate(w["S"])
    assert np.array_equal(Rd.cpu().numpy(), R) and np.array_equal(Sd.cpu().numpy(), S)
    got = engine.hash_join(Rd, Sd)
    assert got.shape[0] == len(S)  # every S key matches exactly one R tuple
    same_multiset(got, O.hash_join(R, S))
    assert engine.checksum(got) == O.checksum(O.hash_join(R, S))


@pytest.mark.parametrize("s", ["0.0", "0.75", "1.0"])
def test_c3_shape_reduced(engine, s):
    """Configuration C3's shape (x4 duplicated R keys, Zipf S with 10% absent) at 1/64 size."""
    w = workload("c3_s" + s, scale=6)
    R, S = O.generate(w["R"]), O.generate(w["S"])
    Rd, Sd = engine.generate(w["R"]), engine.generate(w["S"])
    assert np.array_equal(Sd.cpu().numpy(), S)
    got = engine.hash_join(Rd, Sd)
    same_multiset(got, O.hash_join(R, S))


def test_capacity_and_guard(engine):
    rng = np.random.default_rng(3)
    R, S = rel(rng, 5000, 0, 100), rel(rng, 20000, 0, 100, key_base=5000)
    total = len(O.hash_join(R, S))
    cap = total // 3
    guard = 1000
    out = torch.full((cap + guard, 4), -7, dtype=torch.int32, device="cuda")
    with pytest.raises(JoinError) as ei:
        engine.hash_join(dev(R), dev(S), out=out[:cap])
    assert ei.value.status == native.EJ_ERR_CAPACITY
    assert torch.all(out[cap:] == -7)  # nothing written past out_cap
    assert engine.count("hash", dev(R), dev(S)) == total


@pytest.mark.parametrize("pb", [-1, 0, 6])
def test_count_then_join_writes_from_the_count(engine, pb):
    """ej_hash_join_count then ej_hash_join on the same relations, as the
    reference sizes its output (hj.cc:997-1115): the join writes from the
    count's table, partitioned S and run descriptors (one launch); a write cut
    short by the capacity keeps them for the retry; any other call that lays
    out the handle's scratch drops them, and the join then runs whole."""
    rng = np.random.default_rng(50 + pb)
    R, S = rel(rng, 50000, 0, 30000), rel(rng, 200003, 0, 40000, key_base=50000)
    ref = O.hash_join(R, S)
    Rd, Sd = dev(R), dev(S)
    engine.set_option("partition_bits", pb)
    try:
        n = engine.count("hash", Rd, Sd)
        assert n == len(ref)
        out = torch.full((n + 64, 4), -7, dtype=torch.int32, device="cuda")
        before = engine.kernel_launches()
        with pytest.raises(JoinError) as ei:
            engine.hash_join(Rd, Sd, out=out[: n // 2])
        assert ei.value.status == native.EJ_ERR_CAPACITY
        assert torch.all(out[n // 2:] == -7)
        got = engine.hash_join(Rd, Sd, out=out[:n])
        assert engine.kernel_launches() - before == 2  # two write passes, nothing rebuilt
        same_multiset(got, ref)
        assert torch.all(out[n:] == -7)
        # the kept count is spent: the next join runs whole
        before = engine.kernel_launches()
        same_multiset(engine.hash_join(Rd, Sd, out=out[:n]), ref)
        assert engine.kernel_launches() - before > 1
        # another call in between drops the kept count
        assert engine.count("hash", Rd, Sd) == n
        engine.exclusive_scan_u32(torch.ones(1000, dtype=torch.int32, device="cuda"))
        before = engine.kernel_launches()
        same_multiset(engine.hash_join(Rd, Sd, out=out[:n]), ref)
        assert engine.kernel_launches() - before > 1
        # as does a count of other relations
        assert engine.count("hash", Rd, Sd[:1000]) == len(O.hash_join(R, S[:1000]))
        same_multiset(engine.hash_join(Rd, Sd, out=out[:n]), ref)
    finally:
        engine.set_option("partition_bits", -1)


@pytest.mark.parametrize("shape", ["three_keys", "hot_keys", "long_runs"])
def test_msd_table_build_skew(engine, shape):
    """Tables of 2^20 rows and more are sorted by two MSD passes and one
    shared-memory sort per 16-bit hash bucket.  Skewed tables take its other
    paths: buckets too large for shared memory (sorted through global memory:
    three keys, or hot keys among unique ones), and sub-buckets longer than one
    thread's insertion sort (runs of 40 to 3000 rows of one key)."""
    rng = np.random.default_rng({"three_keys": 1, "hot_keys": 2, "long_runs": 3}[shape])
    n = (1 << 20) + 333
    if shape == "three_keys":
        vals = rng.integers(5, 8, n)
        S = rel(rng, 20, 4, 9, key_base=n)
    else:
        vals = rng.choice(1 << 30, size=n, replace=False)
        if shape == "hot_keys":
            hot = rng.choice(1 << 30, size=40, replace=False)
            vals[: n // 5] = hot[rng.integers(0, 40, n // 5)]
            skewed = vals[: n // 5]
        else:
            runs = rng.integers(40, 3000, 60)
            pos = np.cumsum(np.concatenate([[0], runs]))
            for i in range(60):
                vals[pos[i]:pos[i + 1]] = vals[pos[i]]
            skewed = vals[: pos[-1]]
        S = np.empty((1 << 18, 2), dtype=np.int32)
        S[:, 0] = np.arange(n, n + len(S))
        S[:, 1] = vals[rng.integers(0, n, len(S))]
        S[: len(S) // 8, 1] = rng.integers(0, 1 << 30, len(S) // 8)
        # the skewed keys only in S rows 0..7; elsewhere 12345 replaces them
        # (a key R holds once at most), so the result stays small
        S[8:, 1] = np.where(np.isin(S[8:, 1], skewed), 12345, S[8:, 1])
        S[:8, 1] = skewed[:8]
    R = np.stack([np.arange(n), vals], axis=1).astype(np.int32)
    R = R[rng.permutation(n)]
    ref = O.hash_join(R, S)
    same_multiset(engine.join("hash", dev(R), dev(S)), ref)
    same_multiset(engine.join("hash_index", dev(R), dev(S)), ref)


@pytest.mark.parametrize("n,dup,s_rows", [(1 << 22, 1, 1 << 23), (1 << 22, 3, 1 << 23), (1 << 20, 1, 17 << 20)])
def test_directory_or_buckets(engine, n, dup, s_rows):
    """A 2^22-row table keeps its key directory when its runs average two rows
    or more (else its build switches to bucket bounds); a 2^20-row table has
    one when the probe side is 16 times its size or more.  Every case must give
    the oracle's rows."""
    rng = np.random.default_rng(40 + dup)
    keys = rng.choice(1 << 24, size=n // dup + 1, replace=False).astype(np.int32)
    R = np.stack([np.arange(n, dtype=np.int32), np.repeat(keys, dup)[:n]], axis=1)
    R = R[rng.permutation(n)]
    S = rel(rng, s_rows, 0, 1 << 24, key_base=n)
    S[: s_rows // 2, 1] = keys[rng.integers(0, len(keys), s_rows // 2)]
    same_multiset(engine.join("hash", dev(R), dev(S)), O.hash_join(R, S))
    if s_rows < (4 << 20):
        same_multiset(engine.join("left_outer", dev(R), dev(S)), O.left_outer_join(R, S))
        same_multiset(engine.join("hash_index", dev(R), dev(S)), O.hash_index_join(R, S))


def test_wide_buckets(engine):
    """Two outliers stretch the value range, so a sorted index's value buckets
    hold tens of thousands of distinct vals (runs found by binary search past
    the first 8 values of a bucket); the same relation in a hash table."""
    rng = np.random.default_rng(21)
    R = rel(rng, 50000, 0, 50000)
    R[0, 1], R[1, 1] = INT_MIN, INT_MAX
    R[2:400, 1] = 777  # one long run inside the dense cluster
    S = rel(rng, 60000, -10, 50010, key_base=50000)
    S[:5, 1] = [INT_MIN, INT_MAX, 777, INT_MIN + 1, INT_MAX - 1]
    for algo in ("sort_index", "hash_index", "hash", "left_outer"):
        same_multiset(engine.join(algo, dev(R), dev(S)), ORACLE[algo](R, S))


def test_index_reuse_and_count(engine):
    rng = np.random.default_rng(5)
    R = rel(rng, 40000, 0, 20000)
    S1, S2 = rel(rng, 100000, 0, 30000, key_base=40000), rel(rng, 7777, -5, 25000, key_base=140000)
    for kind, ref in (("hash", O.hash_index_join), ("sort", O.sort_index_join)):
        ix = engine.build_index(kind, dev(R))
        try:
            same_multiset(ix.join(dev(S1)), ref(R, S1))
            same_multiset(ix.join(dev(S2)), ref(R, S2))
            assert ix.count(dev(S1)) == len(ref(R, S1))
            same_multiset(ix.left_outer_join(dev(S2)), O.left_outer_join(R, S2))
        finally:
            ix.free()


@pytest.mark.parametrize("case", [0, 1, 2, 4, 6, 7])
def test_sort_index_merge_join(engine, case):
    """The merge join of a sort index with S in value order gives the oracle's
    rows, whether the call sorts S or the caller passes it sorted."""
    nR, nS, (lo, hi) = CASES[case]
    rng = np.random.default_rng(300 + case)
    R, S = rel(rng, nR, lo, hi), rel(rng, nS, lo, hi, key_base=nR)
    ref = O.sort_index_join(R, S)
    ix = engine.build_index("sort", dev(R))
    try:
        same_multiset(ix.merge_join(dev(S)), ref)
        order = np.argsort(S[:, 1], kind="stable")
        same_multiset(ix.merge_join(dev(S[order]), s_sorted=True), ref)
        if len(ref) > 2:  # capacity: the count, nothing written past out_cap
            out = torch.full((len(ref) // 2 + 16, 4), -5, dtype=torch.int32, device="cuda")
            with pytest.raises(JoinError) as ei:
                ix.merge_join(dev(S), out=out[: len(ref) // 2])
            assert ei.value.status == native.EJ_ERR_CAPACITY
            assert torch.all(out[len(ref) // 2:] == -5)
    finally:
        ix.free()
    hx = engine.build_index("hash", dev(R))
    try:
        with pytest.raises(JoinError) as ei:
            hx.merge_join(dev(S))
        assert ei.value.status == native.EJ_ERR_INVALID
    finally:
        hx.free()


def test_star_join(engine):
    w = workload("c4_star", scale=8)
    t = {k: O.generate(v) for k, v in w.items()}
    got = engine.star_join3(*(dev(t[k]) for k in ("F1", "F2", "D1", "D2")))
    ref = O.star_join3(t["F1"], t["F2"], t["D1"], t["D2"])
    assert len(ref) == len(t["F1"])  # 100% foreign-key hits, unique dimension keys
    same_multiset(got, ref)
    # many-to-many dimensions
    rng = np.random.default_rng(9)
    F1, F2 = rel(rng, 3000, 0, 50), rel(rng, 3000, 0, 40)
    F2[:, 0] = F1[:, 0]
    D1, D2 = rel(rng, 200, 0, 60), rel(rng, 300, 0, 45)
    same_multiset(engine.star_join3(dev(F1), dev(F2), dev(D1), dev(D2)), O.star_join3(F1, F2, D1, D2))


def test_host_buffer_path(engine):
    rng = np.random.default_rng(21)
    R, S = rel(rng, 30000, 0, 50000), rel(rng, 90000, 0, 60000, key_base=30000)
    ref = O.hash_join(R, S)
    out = np.zeros((len(ref) + 10, 4), dtype=np.int32)
    n = engine.join_host("hash", R, S, out)
    assert n == len(ref)
    assert np.array_equal(O.canon(out[:n]), O.canon(ref))


def test_async_hash_join(engine):
    rng = np.random.default_rng(22)
    R, S = rel(rng, 20000, 0, 30000), rel(rng, 80000, 0, 30000, key_base=20000)
    ref = O.hash_join(R, S)
    out = torch.empty((len(ref), 4), dtype=torch.int32, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    engine.hash_join_async(dev(R), dev(S), out, d_count)
    assert engine.sync_status() == native.EJ_OK
    assert int(d_count.item()) == len(ref)
    same_multiset(out, ref)


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 1 << 20, 3_000_001])
def test_exclusive_scan(engine, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    got = engine.exclusive_scan_u32(torch.from_numpy(x.view(np.int32)).cuda()).cpu().numpy().view(np.uint64)
    ref = np.zeros(n + 1, dtype=np.uint64)
    ref[1:] = np.cumsum(x.astype(np.uint64))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", ["c1", "c2", "c3_s0.0", "c3_s0.75", "c3_s1.0", "c4", "c4_star"])
def test_device_generator_matches_host(engine, name):
    for side, spec in workload(name, scale=8).items():
        assert np.array_equal(engine.generate(spec).cpu().numpy(), O.generate(spec)), (name, side)


def test_checksum_matches_oracle(engine):
    rng = np.random.default_rng(4)
    rows = rng.integers(INT_MIN, INT_MAX, size=(100003, 4), dtype=np.int64).astype(np.int32)
    assert engine.checksum(dev(rows)) == O.checksum(rows)
    star = rng.integers(INT_MIN, INT_MAX, size=(5001, 8), dtype=np.int64).astype(np.int32)
    assert engine.checksum(dev(star)) == O.checksum(star)


def test_bnl_c2_shape_reduced(engine):
    w = workload("c2", scale=2)
    R, S = O.generate(w["R"]), O.generate(w["S"])
    got = engine.join("bnl", dev(R), dev(S))
    same_multiset(got, O.hash_join(R, S))
    assert engine.count("bnl", dev(R), dev(S)) == len(got)


def test_bnl_unaligned_probe_side(engine):
    """S not 16-byte aligned takes the plain-load staging path instead of TMA."""
    rng = np.random.default_rng(8)
    R, S = rel(rng, 5000, 0, 3000), rel(rng, 20001, 0, 3000, key_base=5000)
    Sd = dev(np.concatenate([np.zeros((1, 2), np.int32), S]))[1:]
    assert Sd.data_ptr() % 16 == 8
    same_multiset(engine.join("bnl", dev(R), Sd), O.bnl_join(R, S))


@pytest.mark.parametrize("case", ["dir_unaligned_probes", "dir_partial_tiles", "buckets_by_header", "dir_long_runs"])
def test_count_pass_over_a_packed_directory(engine, case):
    """The count pass of a packed key directory takes two 128-probe tiles per
    warp with 16-byte probe loads and stores each probe's directory entry as
    its run descriptor; a probe side not 16-byte aligned, a last warp with
    partial tiles, and a directory table whose build chose bucket bounds
    (unique keys: the header's bits = 0) take its general path; a table of a
    few long runs (40 keys) takes the escape of runs of 31 rows or more.
    Count, then the write from the count's descriptors, against the oracle."""
    rng = np.random.default_rng({"dir_unaligned_probes": 61, "dir_partial_tiles": 62, "buckets_by_header": 63,
                                 "dir_long_runs": 64}[case])
    if case == "dir_long_runs":  # 40 keys of about 1250 rows each
        R = rel(rng, 50000, 0, 40)
        S = rel(rng, 4000, -5, 45, key_base=50000)
    elif case == "buckets_by_header":
        nR = 1 << 23  # the planner's class: a directory table; unique keys: bucket bounds
        R = np.stack([np.arange(nR), rng.permutation(nR)], axis=1).astype(np.int32)
        S = rel(rng, (1 << 20) + 77, 0, 2 * nR, key_base=nR)
    else:
        R = rel(rng, 60000, 0, 20000)  # runs of about three rows
        S = rel(rng, 300077, 0, 30000, key_base=60000)  # 300077 = 1172 x 256 + 45
    ref = O.hash_join(R, S)
    Rd = dev(R)
    if case == "dir_unaligned_probes":  # rows 8 bytes past a 16-byte boundary, probed in place
        Sd = dev(np.vstack([np.zeros((1, 2), np.int32), S]))[1:]
        assert Sd.data_ptr() % 16 == 8
    else:
        Sd = dev(S)
    try:
        if case != "buckets_by_header":
            engine.set_option("table", native.EJ_TABLE_FORMAT_DIRECTORY)
        if case == "dir_unaligned_probes":
            engine.set_option("partition_bits", 0)
        n = engine.count("hash", Rd, Sd)
        assert n == len(ref)
        out = torch.full((n + 16, 4), -7, dtype=torch.int32, device="cuda")
        same_multiset(engine.hash_join(Rd, Sd, out=out[:n]), ref)
        assert torch.all(out[n:] == -7)
    finally:
        engine.set_option("table", 0)
        engine.set_option("partition_bits", -1)
