"""Full-size joins against the oracle's digests (count + order-independent checksum).

The configurations the bench measures are checked here at their full sizes:
the three skewed 2^26 x 2^28 hash joins (up to 9.7e8 result rows, 15.5 GB
each, past 2^32 output bytes) and the 2^24 x 2^26 index, outer and star
joins.  Their results are too large for the oracle to materialise, so
tests/golden/fullsize.json holds the oracle's count and checksum of each
(tests/golden/make_fullsize.py: relations generated on the host with the
same seeded generators, joined by the multithreaded restatement of
joins/multi_joins/hash, every row fed to the checksum).  The inputs here come
from the device generators and the checksum from ej_checksum, the same
function as the oracle's; equal digests mean equal result multisets up to a
64-bit checksum collision.  Integer joins: no tolerance.
"""
import pytest
import torch

from eating_one_gb300.workloads import workload
from tests import golden

pytestmark = pytest.mark.gpu

GOLD = golden.fullsize()


def digest(engine, rows: torch.Tensor) -> dict:
    return {"count": int(rows.shape[0]), "checksum": engine.checksum(rows)}


@pytest.mark.parametrize("name", ["c3_s0.0", "c3_s0.75", "c3_s1.0"])
def test_c3_full_size(engine, name):
    w = workload(name)
    R, S = engine.generate(w["R"]), engine.generate(w["S"])
    want = GOLD[name]["inner"]
    # the reference's sequence: the count sizes the output, the join writes it
    # (the write reuses the count's table, partitioned S and run descriptors)
    n = engine.count("hash", R, S)
    assert n == want["count"]
    out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    assert digest(engine, engine.hash_join(R, S, out=out)) == want
    # one call without a count: table build, S partition and the one-pass probe
    out.fill_(0)
    assert digest(engine, engine.hash_join(R, S, out=out)) == want
    del out
    torch.cuda.empty_cache()


def test_c4_index_joins_full_size(engine):
    w = workload("c4")
    R, S = engine.generate(w["R"]), engine.generate(w["S"])
    want = GOLD["c4"]["inner"]
    out = torch.empty((want["count"], 4), dtype=torch.int32, device="cuda")
    for kind in ("hash", "sort"):
        ix = engine.build_index(kind, R)
        try:
            assert ix.count(S) == want["count"], kind
            out.fill_(0)
            assert digest(engine, ix.join(S, out=out)) == want, kind
            if kind == "sort":  # the merge join, S sorted by the call
                out.fill_(0)
                assert digest(engine, ix.merge_join(S, out=out)) == want
        finally:
            ix.free()
    for algo in ("hash_index", "sort_index", "hash"):
        out.fill_(0)
        assert digest(engine, engine.join(algo, R, S, out=out)) == want, algo


def test_c4_left_outer_full_size(engine):
    w = workload("c4")
    R, S = engine.generate(w["R"]), engine.generate(w["S"])
    want = GOLD["c4"]["outer"]
    assert engine.count("left_outer", R, S) == want["count"]
    assert digest(engine, engine.join("left_outer", R, S)) == want
    ix = engine.build_index("hash", R)
    try:
        assert digest(engine, ix.left_outer_join(S)) == want
    finally:
        ix.free()


def test_c4_star_full_size(engine):
    w = workload("c4_star")
    t = {k: engine.generate(v) for k, v in w.items()}
    rows = engine.star_join3(t["F1"], t["F2"], t["D1"], t["D2"])
    assert digest(engine, rows) == GOLD["c4_star"]["star"]
