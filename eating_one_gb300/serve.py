"""Python mirror of the request server (ej_server_* in include/ej.h) and the
served-stream workload (configuration C5).

C5: join requests with |R| = floor(2^(10 + 12U)) (log-uniform in [2^10, 2^22]),
|S| = 4|R|, R = |R| distinct keys from [0, |R|u), S uniform over [0, |R|u),
u in {1, 2, 8} (match rates 100/50/12.5%), Poisson arrivals.  The stream is
drawn from a pool of request instances generated on the device once, so the
timed region contains serving work only.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import torch

from . import native
from .engine import Engine, JoinError
from .workloads import EJ_GEN_PERM, EJ_GEN_UNIFORM, make_spec

BATCHED, PER_JOIN = native.EJ_SERVE_BATCHED, native.EJ_SERVE_PER_JOIN


class Server:
    def __init__(self, mode: int, device: int = 0, lanes: int = 2, max_batch_joins: int = 1024,
                 lane_bytes: int = 16 << 30, max_queued: int = 0, checksums: bool = False):
        """checksums: every completion carries the device-computed checksum of
        its request's rows (EJ_SERVE_CHECKSUM)."""
        self.lib = native.load()
        self.checksums = checksums
        cfg = native.ServerConfig(device, mode, lanes, max_batch_joins, lane_bytes, max_queued,
                                  native.EJ_SERVE_CHECKSUM if checksums else 0)
        h = C.c_void_p()
        st = self.lib.ej_server_create(C.byref(cfg), C.byref(h))
        if st != native.EJ_OK:
            raise JoinError(st, "ej_server_create failed")
        self.h = h

    def now_ns(self) -> int:
        return int(self.lib.ej_now_ns())

    def submit(self, desc: native.JoinDesc, tag: int, arrival_ns: int = 0) -> None:
        st = self.lib.ej_server_submit(self.h, C.byref(desc), tag, arrival_ns)
        if st != native.EJ_OK:
            raise JoinError(st, "ej_server_submit failed")

    def poll(self, max_n: int = 4096, wait_us: int = 0) -> list[native.Completion]:
        buf = (native.Completion * max_n)()
        n = C.c_uint32(0)
        self.lib.ej_server_poll(self.h, buf, max_n, C.byref(n), wait_us)
        return [buf[i] for i in range(n.value)]

    def drain(self) -> None:
        self.lib.ej_server_drain(self.h)

    def close(self) -> None:
        if self.h:
            self.lib.ej_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RequestPool:
    """Device-resident request instances of the C5 stream with their output buffers.

    copies > 1: every instance gets that many output buffers, each exactly as
    large as its result (the stream's request i writes into buffer slot
    i % (instances * copies)), so that requests of one instance in flight at
    once write to different buffers - needed when every result is verified by
    its checksum.  checksums: also record each instance's result checksum (its
    rows joined alone, ej_single_hash_join)."""

    def __init__(self, engine: Engine, n_instances: int, seed: int = 0xE1A00005, lo_bits: float = 10.0,
                 hi_bits: float = 22.0, copies: int = 1, checksums: bool = False):
        rng = np.random.default_rng(seed)
        self.ninst = n_instances
        self.R, self.S, self.out, self.desc, self.u = [], [], [], [], []
        for i in range(n_instances):
            nR = int(np.floor(2.0 ** (lo_bits + (hi_bits - lo_bits) * rng.random())))
            u = int(rng.choice([1, 2, 8]))
            d = nR * u
            self.R.append(engine.generate(make_spec(EJ_GEN_PERM, nR, d, seed * 7 + 2 * i, seed * 7 + 2 * i + 1)))
            self.S.append(engine.generate(make_spec(EJ_GEN_UNIFORM, 4 * nR, d, seed * 11 + i)))
            self.u.append(u)
        torch.cuda.synchronize()
        self.expected = [engine.count("hash", R, S) for R, S in zip(self.R, self.S)]
        self.expected_sum = [engine.checksum(engine.join("single_hash", R, S)) if checksums else None
                             for R, S in zip(self.R, self.S)]
        for c in range(copies):
            for i in range(n_instances):
                R, S = self.R[i], self.S[i]
                # every S row matches at most once (unique R keys): 4|R| rows hold any result
                cap = 4 * R.shape[0] if copies == 1 else max(self.expected[i], 1)
                out = torch.empty((cap, 4), dtype=torch.int32, device=engine.device)
                self.out.append(out)
                self.desc.append(native.JoinDesc(R.data_ptr(), R.shape[0], S.data_ptr(), S.shape[0],
                                                 out.data_ptr(), cap))

    def tuples(self, i: int) -> int:
        """Input tuples of request i (instance i % instances)."""
        k = i % self.ninst
        return self.R[k].shape[0] + self.S[k].shape[0]


def run_stream(server: Server, pool: RequestPool, n_requests: int, rate_per_s: float | None, seed: int = 1) -> dict:
    """Submit n_requests (instance i % pool size) with Poisson arrivals at rate_per_s
    (None: all at once); returns latency percentiles and throughput."""
    rng = np.random.default_rng(seed)
    k = len(pool.desc)
    gaps = rng.exponential(1.0 / rate_per_s, n_requests) if rate_per_s else np.zeros(n_requests)
    comps: list = []
    done = threading.Event()

    def collector():
        got = 0
        while got < n_requests:
            c = server.poll(4096, wait_us=2000)
            comps.extend(c)
            got += len(c)
        done.set()

    th = threading.Thread(target=collector, daemon=True)
    th.start()
    t0 = server.now_ns() + 2_000_000
    arrivals = t0 + np.cumsum(gaps * 1e9).astype(np.int64)
    for i in range(n_requests):
        a = int(arrivals[i])
        while True:
            now = server.now_ns()
            if now >= a:
                break
            if a - now > 200_000:
                time.sleep((a - now - 100_000) / 1e9)
        server.submit(pool.desc[i % k], i, a)
    done.wait()
    th.join()
    n = pool.ninst
    bad = [c.tag for c in comps if c.status != native.EJ_OK or c.count != pool.expected[c.tag % n] or
           (server.checksums and c.checksum != pool.expected_sum[c.tag % n])]
    lat = np.array([c.done_ns - c.arrival_ns for c in comps], dtype=np.float64) / 1e6
    first = min(c.arrival_ns for c in comps)
    last = max(c.done_ns for c in comps)
    tuples = sum(pool.tuples(c.tag) for c in comps)
    return {"requests": n_requests, "rate_per_s": rate_per_s, "checked": "checksum" if server.checksums else "count",
            "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_batch": float(np.mean([c.batch_joins for c in comps])),
            "seconds": (last - first) / 1e9, "tuples_per_s": tuples / ((last - first) / 1e9),
            "requests_per_s": n_requests / ((last - first) / 1e9), "wrong": len(bad)}
