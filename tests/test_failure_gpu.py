"""Failure paths, driven from the host: no test here faults, traps or hangs a GPU.

- Bounded device waits: the handle's wait limit (EJ_OPT_WAIT_LIMIT_NS) set to
  0 makes the look-back scan and the nested loop's copy waits give up at the
  first unmet poll; the call returns EJ_ERR_TIMEOUT, and with the default
  limit restored the same handle gives correct results again.
- Allocation failure: ej_inject_alloc_failures makes the library's next
  allocations fail as if memory were exhausted (handle creation, scratch
  growth, index storage, server lanes, host-buffer staging); each call
  returns EJ_ERR_NOMEM and the next one succeeds.
- Admission: a server whose queue holds at most a few requests refuses
  submits past it with EJ_ERR_BUSY; the accepted requests complete with
  their correct counts, the refused ones never complete.
The reference has none of this: its drivers exit(1) after any failed call
(joins/hashJoin_gpu/main_street/hj.cc:213-227, :467-475).
"""
import ctypes as C

import numpy as np
import pytest
import torch

from eating_one_gb300 import native
from eating_one_gb300.engine import Engine, JoinError
from eating_one_gb300.serve import BATCHED, RequestPool, Server
from eating_one_gb300.workloads import workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def expect_status(status, fn, *args, **kw):
    with pytest.raises(JoinError) as ei:
        fn(*args, **kw)
    assert ei.value.status == status, ei.value


def scan_ref(x: np.ndarray) -> np.ndarray:
    ref = np.zeros(len(x) + 1, dtype=np.uint64)
    ref[1:] = np.cumsum(x.astype(np.uint64))
    return ref


def test_scan_wait_limit_runs_out(engine):
    n = 1 << 24
    x = torch.ones(n, dtype=torch.int32, device="cuda")
    engine.set_option("wait_limit_ns", 0)
    try:
        # 4096 tiles in flight at once: some tile finds a predecessor that has
        # not published yet and gives up at once
        timed_out = False
        for _ in range(5):
            try:
                engine.exclusive_scan_u32(x)
            except JoinError as e:
                assert e.status == native.EJ_ERR_TIMEOUT, e
                timed_out = True
                break
        assert timed_out
    finally:
        engine.set_option("wait_limit_ns", -1)
    got = engine.exclusive_scan_u32(x).cpu().numpy().view(np.uint64)
    assert np.array_equal(got, scan_ref(np.ones(n, dtype=np.uint32)))


def test_nested_loop_wait_limit_runs_out(engine):
    w = workload("c2", scale=2)
    R, S = engine.generate(w["R"]), engine.generate(w["S"])
    assert S.data_ptr() % 16 == 0  # the copy-engine (TMA) path, whose waits are bounded
    engine.set_option("wait_limit_ns", 0)
    try:
        # every CTA waits for its first S tile right after issuing its copy
        expect_status(native.EJ_ERR_TIMEOUT, engine.count, "bnl", R, S)
        expect_status(native.EJ_ERR_TIMEOUT, engine.join, "bnl", R, S,
                      out=torch.empty((1 << 20, 4), dtype=torch.int32, device="cuda"))
    finally:
        engine.set_option("wait_limit_ns", -1)
    ref = O.bnl_join(R.cpu().numpy(), S.cpu().numpy())
    got = engine.join("bnl", R, S)
    assert np.array_equal(O.canon(got.cpu().numpy()), O.canon(ref))


def test_wait_limit_option_range(engine):
    for bad in (-2, 10 ** 10 + 1):
        expect_status(native.EJ_ERR_INVALID, engine.set_option, "wait_limit_ns", bad)
    engine.set_option("wait_limit_ns", 10 ** 10)
    engine.set_option("wait_limit_ns", -1)


def test_create_fails_when_allocation_fails():
    lib = native.load()
    for k in range(1, 5):  # each of the handle's four allocations in turn
        lib.ej_inject_alloc_failures(k)
        h = C.c_void_p()
        try:
            # the first k - 1 allocations succeed only if the injected count is
            # used up first, so every k fails at its first allocation
            assert lib.ej_create(0, C.byref(h)) == native.EJ_ERR_NOMEM
            assert not h.value
        finally:
            lib.ej_inject_alloc_failures(0)
    h = C.c_void_p()
    assert lib.ej_create(0, C.byref(h)) == native.EJ_OK
    assert lib.ej_destroy(h) == native.EJ_OK


def test_join_index_and_host_paths_fail_cleanly():
    rng = np.random.default_rng(3)
    Rn = np.stack([np.arange(20000), rng.integers(0, 9000, 20000)], axis=1).astype(np.int32)
    Sn = np.stack([np.arange(70000), rng.integers(0, 9000, 70000)], axis=1).astype(np.int32)
    ref = O.canon(O.hash_join(Rn, Sn))
    lib = native.load()
    with Engine(0) as e:
        R, S = torch.from_numpy(Rn).cuda(), torch.from_numpy(Sn).cuda()
        try:
            # scratch growth (a fresh handle has none)
            lib.ej_inject_alloc_failures(1)
            expect_status(native.EJ_ERR_NOMEM, e.join, "hash", R, S)
            lib.ej_inject_alloc_failures(0)
            assert np.array_equal(O.canon(e.join("hash", R, S).cpu().numpy()), ref)
            # index storage
            lib.ej_inject_alloc_failures(1)
            expect_status(native.EJ_ERR_NOMEM, e.build_index, "hash", R)
            lib.ej_inject_alloc_failures(0)
            ix = e.build_index("hash", R)
            try:
                assert np.array_equal(O.canon(ix.join(S).cpu().numpy()), ref)
            finally:
                ix.free()
            # host-buffer staging and the chunked pipeline's buffers
            out = np.zeros((len(ref), 4), dtype=np.int32)
            for algo_call in (lambda: e.join_host("hash", Rn, Sn, out),
                              lambda: e.join_host_chunked("hash", Rn, Sn, out, s_chunk=1 << 14)):
                e.trim()
                lib.ej_inject_alloc_failures(1)
                expect_status(native.EJ_ERR_NOMEM, algo_call)
                lib.ej_inject_alloc_failures(0)
                out.fill(0)
                assert algo_call() == len(ref)
                assert np.array_equal(O.canon(out), ref)
        finally:
            lib.ej_inject_alloc_failures(0)


def test_server_create_fails_when_allocation_fails():
    lib = native.load()
    lib.ej_inject_alloc_failures(1)
    try:
        expect_status(native.EJ_ERR_NOMEM, Server, BATCHED, lanes=2)
    finally:
        lib.ej_inject_alloc_failures(0)
    Server(BATCHED, lanes=1).close()


def test_server_refuses_past_its_queue_limit(engine):
    pool = RequestPool(engine, 8, seed=123, lo_bits=18, hi_bits=20)
    srv = Server(BATCHED, lanes=1, max_batch_joins=2, max_queued=3)
    accepted, refused = [], 0
    try:
        t = srv.now_ns()
        for i in range(400):
            d = pool.desc[i % len(pool.desc)]
            st = srv.lib.ej_server_submit(srv.h, C.byref(d), i, t)
            if st == native.EJ_ERR_BUSY:
                refused += 1
            else:
                assert st == native.EJ_OK
                accepted.append(i)
        srv.drain()
        comps = srv.poll(1000)
    finally:
        srv.close()
    assert refused > 0 and accepted
    assert sorted(c.tag for c in comps) == accepted
    for c in comps:
        assert c.status == native.EJ_OK
        assert c.count == pool.expected[c.tag % len(pool.desc)]
