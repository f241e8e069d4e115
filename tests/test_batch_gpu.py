"""Batched hash joins: every join of a mixed batch gives the rows it gives
alone (ej_single_hash_join; compared as multisets, bit for bit), and the
oracle's result multiset."""
import numpy as np
import pytest
import torch

from eating_one_gb300 import native
from eating_one_gb300.engine import JoinError
from eating_one_gb300.workloads import EJ_GEN_PERM, EJ_GEN_UNIFORM, make_spec
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def request(engine, i: int, nR: int, u: int):
    """A served-stream request: |R| distinct keys from [0, |R|u), |S| = 4|R| uniform over it."""
    d = max(nR * u, 1)
    R = engine.generate(make_spec(EJ_GEN_PERM, nR, d, 1000 + i, 77 + i)) if nR else torch.zeros(
        (0, 2), dtype=torch.int32, device="cuda")
    S = engine.generate(make_spec(EJ_GEN_UNIFORM, 4 * nR, d, 5000 + i)) if nR else torch.zeros(
        (7, 2), dtype=torch.int32, device="cuda")
    return R, S


def test_batch_equals_alone_and_oracle(engine):
    rng = np.random.default_rng(3)
    sizes = [int(2 ** rng.uniform(10, 17)) for _ in range(23)] + [1, 3, 8191, 8192, 8193, 0]
    pairs = [request(engine, i, n, [1, 2, 8][i % 3]) for i, n in enumerate(sizes)]
    got = engine.batch_hash_join(pairs)
    for (R, S), rows in zip(pairs, got):
        alone = engine.join("single_hash", R, S)
        assert np.array_equal(O.canon(rows.cpu().numpy()), O.canon(alone.cpu().numpy()))  # the same rows
        ref = O.hash_join(R.cpu().numpy(), S.cpu().numpy())
        assert np.array_equal(O.canon(rows.cpu().numpy()), O.canon(ref))


def test_batch_duplicates_and_capacity(engine):
    rng = np.random.default_rng(4)
    pairs = []
    for i in range(5):
        nR, nS = int(rng.integers(100, 5000)), int(rng.integers(100, 20000))
        R = np.stack([np.arange(nR), rng.integers(-50, 50, nR)], 1).astype(np.int32)
        S = np.stack([np.arange(nS), rng.integers(-60, 60, nS)], 1).astype(np.int32)
        pairs.append((torch.from_numpy(R).cuda(), torch.from_numpy(S).cuda()))
    got = engine.batch_hash_join(pairs)
    for (R, S), rows in zip(pairs, got):
        ref = O.hash_join(R.cpu().numpy(), S.cpu().numpy())
        assert np.array_equal(O.canon(rows.cpu().numpy()), O.canon(ref))
    # one join with too small an output: EJ_ERR_CAPACITY, nothing written past its end
    outs = [torch.full((max(r.shape[0], 1) + 64, 4), -9, dtype=torch.int32, device="cuda") for r in got]
    small = got[2].shape[0] // 2
    outs[2] = torch.full((small + 64, 4), -9, dtype=torch.int32, device="cuda")
    views = [o[: max(r.shape[0], 1)] for o, r in zip(outs, got)]
    views[2] = outs[2][:small]
    with pytest.raises(JoinError) as ei:
        engine.batch_hash_join(pairs, outs=views)
    assert ei.value.status == native.EJ_ERR_CAPACITY
    assert torch.all(outs[2][small:] == -9)


def test_batch_with_large_joins(engine):
    """Joins of 2^20 R rows and more in a batch (four segmented LSD passes
    over every join's R, an in-place probe): mixed with small and medium ones
    they give the same rows as alone, and a large one with too small an
    output reports EJ_ERR_CAPACITY without writing past its end."""
    sizes = [1 << 20, 700, 3000, (1 << 20) + 5, 40000, 1 << 21]
    pairs = [request(engine, 100 + i, n, [1, 2, 8][i % 3]) for i, n in enumerate(sizes)]
    got = engine.batch_hash_join(pairs)
    for (R, S), rows in zip(pairs, got):
        alone = engine.join("single_hash", R, S)
        assert np.array_equal(O.canon(rows.cpu().numpy()), O.canon(alone.cpu().numpy()))
    ref = O.hash_join(pairs[3][0].cpu().numpy(), pairs[3][1].cpu().numpy())
    assert np.array_equal(O.canon(got[3].cpu().numpy()), O.canon(ref))
    outs = [torch.full((max(r.shape[0], 1) + 64, 4), -9, dtype=torch.int32, device="cuda") for r in got]
    views = [o[: max(r.shape[0], 1)] for o, r in zip(outs, got)]
    small = got[0].shape[0] // 2
    views[0] = outs[0][:small]
    with pytest.raises(JoinError) as ei:
        engine.batch_hash_join(pairs, outs=views)
    assert ei.value.status == native.EJ_ERR_CAPACITY
    assert torch.all(outs[0][small:] == -9)
    for k in (1, 2, 3, 4, 5):  # the other joins are whole
        assert np.array_equal(O.canon(views[k][: got[k].shape[0]].cpu().numpy()), O.canon(got[k].cpu().numpy()))
