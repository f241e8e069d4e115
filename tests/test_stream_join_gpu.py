"""Chunked (out-of-core) host-buffer joins against the oracle: R in device
blocks, S streamed in chunks, pinned and pageable host buffers."""
import numpy as np
import pytest

from eating_one_gb300 import native
from eating_one_gb300.engine import JoinError
from eating_one_gb300.workloads import workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rels(name, scale):
    w = workload(name, scale)
    return O.generate(w["R"]), O.generate(w["S"])


def _host(a, pinned):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.pin_memory() if pinned else t


@pytest.mark.parametrize("algo", ["hash", "bnl"])
@pytest.mark.parametrize("pin_in,pin_out", [(True, True), (False, False), (True, False), (False, True)])
@pytest.mark.parametrize("r_block,s_chunk", [(0, 0), (1000, 3000), (5000, 77777)])
@pytest.mark.parametrize("name,scale", [("c1", 6), ("c2", 4)])
def test_matches_oracle(engine, algo, pin_in, pin_out, r_block, s_chunk, name, scale):
    R, S = _rels(name, scale)
    want = O.canon(O.hash_join(R, S))
    out = _host(np.zeros((len(want) + 5, 4), np.int32), pin_out)
    n = engine.join_host_chunked(algo, _host(R, pin_in), _host(S, pin_in), out, r_block, s_chunk)
    assert n == len(want)
    assert np.array_equal(O.canon(out.numpy()[:n]), want)


@pytest.mark.parametrize("algo", ["hash", "bnl"])
@pytest.mark.parametrize("pin_out", [True, False])
def test_capacity(engine, algo, pin_out):
    """Past out_cap rows are counted, not written: the written rows are a
    sub-multiset of the join, the count is the full count."""
    R, S = _rels("c2", 4)
    want = O.canon(O.hash_join(R, S))
    cap = len(want) // 3
    out = _host(np.zeros((cap, 4), np.int32), pin_out)
    n = engine.join_host_chunked(algo, _host(R, True), _host(S, True), out, 1500, 20000)
    assert n == len(want)
    got = O.canon(out.numpy())
    # sub-multiset: every written row, with multiplicity, occurs in the join
    allrows = np.concatenate([want, got])
    u, c = np.unique(allrows, axis=0, return_counts=True)
    uw, cw = np.unique(want, axis=0, return_counts=True)
    assert len(u) == len(uw) and np.all(c <= 2 * cw)


def test_many_blocks_and_chunks_large(engine):
    """2^21 x 2^23 skewed join (about 3*10^7 rows) through 4 R blocks x 4 S chunks,
    rows written straight into pinned host memory."""
    R, S = _rels("c3_s1.0", 5)
    want = O.hash_join(R, S)
    out = _host(np.zeros((len(want), 4), np.int32), True)
    n = engine.join_host_chunked("hash", _host(R, True), _host(S, True), out, len(R) // 4, len(S) // 4)
    assert n == len(want)
    assert O.checksum(out.numpy()) == O.checksum(want)


def test_empty_and_invalid(engine):
    R, S = _rels("c1", 8)
    out = _host(np.zeros((10, 4), np.int32), True)
    assert engine.join_host_chunked("hash", _host(R[:0], True), _host(S, True), out) == 0
    assert engine.join_host_chunked("bnl", _host(R, True), _host(S[:0], True), out) == 0
    with pytest.raises(JoinError) as e:
        engine.join_host_chunked("sort_index", _host(R, True), _host(S, True), out)
    assert e.value.status == native.EJ_ERR_INVALID
