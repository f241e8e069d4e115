"""The request server: every request's result is the same alone and in the mix.

A mixed stream of C5-shaped requests goes through the server in batched and
per-join mode; each request's rows must equal, as a multiset and bit for bit,
the rows of the same join run alone (ej_single_hash_join), and its count the
oracle's count on a sample."""
import numpy as np
import pytest
import torch

from eating_one_gb300 import native
from eating_one_gb300.serve import BATCHED, PER_JOIN, RequestPool, Server, run_stream
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pool(engine):
    return RequestPool(engine, 24, seed=99, lo_bits=10, hi_bits=16)


@pytest.mark.parametrize("mode", [BATCHED, PER_JOIN])
def test_results_same_alone_and_in_mix(engine, pool, mode):
    alone = [engine.join("single_hash", R, S) for R, S in zip(pool.R, pool.S)]
    srv = Server(mode, lanes=2, max_batch_joins=16)
    try:
        for o in pool.out:
            o.fill_(-1)
        t = srv.now_ns()
        for i, d in enumerate(pool.desc):
            srv.submit(d, i, t)
        srv.drain()
        comps = srv.poll(1000)
    finally:
        srv.close()
    assert sorted(c.tag for c in comps) == list(range(len(pool.desc)))
    for c in comps:
        assert c.status == native.EJ_OK
        assert c.count == pool.expected[c.tag] == alone[c.tag].shape[0]
        got = pool.out[c.tag][: c.count]  # the same rows as alone, order unspecified
        assert np.array_equal(O.canon(got.cpu().numpy()), O.canon(alone[c.tag].cpu().numpy()))
    if mode == BATCHED:
        assert max(c.batch_joins for c in comps) > 1
    for i in (0, 5, 17):
        ref = O.hash_join(pool.R[i].cpu().numpy(), pool.S[i].cpu().numpy())
        assert len(ref) == pool.expected[i]


def test_poisson_stream_counts(engine, pool):
    srv = Server(BATCHED, lanes=2, max_batch_joins=64)
    try:
        r = run_stream(srv, pool, 200, rate_per_s=20000.0)
    finally:
        srv.close()
    assert r["wrong"] == 0 and r["p99_ms"] >= r["p50_ms"] > 0


@pytest.mark.parametrize("mode", [BATCHED, PER_JOIN])
def test_served_results_checked_by_checksum(engine, mode):
    """With EJ_SERVE_CHECKSUM every completion carries the checksum of its
    request's rows, computed on the device; each must equal the checksum of
    the same join run alone.  A planted wrong expectation (on the host) is
    caught."""
    pool = RequestPool(engine, 12, seed=5, lo_bits=10, hi_bits=15, copies=3, checksums=True)
    srv = Server(mode, lanes=2, max_batch_joins=16, checksums=True)
    try:
        r = run_stream(srv, pool, 150, None, seed=3)
        assert r["wrong"] == 0 and r["checked"] == "checksum"
        pool.expected_sum[4] ^= 1
        r = run_stream(srv, pool, 36, None, seed=4)
        assert r["wrong"] == 3  # requests 4, 16 and 28
    finally:
        srv.close()
