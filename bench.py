#!/usr/bin/env python3
"""Benchmark of the GB300 join engine on the skewed hash-join workload.

One step = the three hash joins of configuration C3 (R = 2^26 tuples holding
2^24 distinct keys x4, S = 2^28 tuples with Zipf(s) keys over R's keys, 10% of
S from an absent key range, s in {0, 0.75, 1}), each run end to end on the
device as a caller sizing its output does: a count (R table build by two MSD
radix passes, a shared-memory sort per bucket group and a key directory; one
S radix pass; a count pass storing every probe's run descriptor), the count
read back, an output of that size, then the write pass from the count's
descriptors.  Inputs are generated on the device with seeded integer
generators (synthetic data; every input is far larger than the 126 MB L2).

Printed (rank 0, one JSON line):
  value      input tuples/s of the whole job (all ranks), inputs resident in HBM
  e2e        the same metric through ej_join_host_chunked (the C ABI call with
             host buffers: host->device copies of R and S and the device->host
             transfer of every result row inside the timed region), with the
             CPU-GPU link's measured bandwidth and the floor it sets
  roofline   the dominant kernel's algorithmic bytes / its event-timed duration
  join_roofline  algorithmic bytes of the whole join, 24(|R|+|S|) + 16|out|,
             over the step time - the fraction of the HBM roofline
  cpu_baseline   the oracle's restatement of the reference CPU hash join
             (joins/CPU_JOIN/hash_cpu) timed on a 1/16-size sample, rank 0

`--impl reference` times that CPU implementation alone (the reference arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "join input tuples/s and % HBM roofline (bit-exact); batched vs per-launch p50/p99"
UNIT = "tuples/s"
VARIANTS = ["c3_s0.0", "c3_s0.75", "c3_s1.0"]
WORKLOAD = ("C3 skewed hash join x3: R=2^26 (2^24 keys x4) join S=2^28 Zipf(s) over R's keys, "
            "10% absent keys, s in {0, 0.75, 1}; one step = the three joins")


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "of measured"}
    return {"hbm_gbs": 6800.0, "source": "of fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.lines: list[str] = []
        self.dev = device_index

    def start(self):
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(self.dev).uuid)
            ident = ["--id=" + (uuid if uuid.startswith("GPU-") else "GPU-" + uuid)]
        except Exception:
            ident = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi"] + ident + ["--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def link_bandwidth(pinned) -> dict:
    """CPU-GPU link: pinned host-to-device, device-to-host and both at once
    (GB/s), copies of up to 1 GiB between `pinned` (a pinned host tensor) and
    device memory, best of three."""
    import torch

    nbytes = min(pinned.numel() * pinned.element_size(), 1 << 30) // 2
    host = pinned.view(-1).view(torch.uint8)[: 2 * nbytes]
    dev = torch.empty(2 * nbytes, dtype=torch.uint8, device="cuda")
    up, down = torch.cuda.Stream(), torch.cuda.Stream()

    def best(fn):
        t = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            t.append(time.perf_counter() - t0)
        return min(t)

    def h2d():
        with torch.cuda.stream(up):
            dev[:nbytes].copy_(host[:nbytes], non_blocking=True)

    def d2h():
        with torch.cuda.stream(down):
            host[nbytes:].copy_(dev[nbytes:], non_blocking=True)

    t_up, t_down = best(h2d), best(d2h)
    t_both = best(lambda: (h2d(), d2h()))
    del dev
    return {"h2d_gbs": round(nbytes / t_up / 1e9, 1), "d2h_gbs": round(nbytes / t_down / 1e9, 1),
            "both_gbs": round(nbytes / t_both / 1e9, 1)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def aggregate(per_rank_ms: list[float], units_per_rank: float, steps: int) -> tuple[float, float]:
    """Whole-job throughput: the slowest rank's time bounds the job.  Returns
    (units per second over all ranks, ms per step of the slowest rank)."""
    ms = max(per_rank_ms)
    return units_per_rank * len(per_rank_ms) * steps / (ms * steps / 1000.0), ms


def gather_ms(ms: float, dist, device) -> list[float]:
    """Every rank's ms per step (all_gather; works on nccl with a CUDA device
    and on gloo with the CPU).  Single process: [ms]."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [ms]
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    g = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(g, t)
    return [float(x.item()) for x in g]


def _cpu_join_timed(R, S, threads: int) -> tuple[float, int]:
    """One oracle join into a preallocated, already-touched output (the
    reference materialises into a calloc'd result array too); returns
    (seconds, rows).  threads 0: the single-threaded joins/CPU_JOIN/hash_cpu
    restatement; else the pthread joins/multi_joins/hash restatement."""
    import ctypes as C

    import numpy as np

    from oracle import oracle as O

    lib = O.load()
    R = np.ascontiguousarray(R, dtype=np.int32)
    S = np.ascontiguousarray(S, dtype=np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731

    def call(out, cap):
        if threads:
            return lib.ejo_hash_join_mt(p(R), len(R), p(S), len(S), out, cap, 1 << 17, threads)
        return lib.ejo_hash_join(p(R), len(R), p(S), len(S), out, cap, 1 << 20)

    n = int(call(None, 0))
    out = np.ones((max(n, 1), 4), dtype=np.int32)  # touched before the clock starts
    t0 = time.perf_counter()
    m = int(call(p(out), n))
    dt = time.perf_counter() - t0
    assert m == n
    return dt, n


def _cpu_rels(scale: int):
    from eating_one_gb300.workloads import workload
    from oracle import oracle as O

    nt = os.cpu_count() or 1
    return [(O.generate(workload(v, scale)["R"], nt), O.generate(workload(v, scale)["S"], nt)) for v in VARIANTS]


def cpu_baseline_sample(scale: int = 4, rels=None) -> dict:
    """The oracle's hash_cpu restatement, single-threaded as the reference
    runs it, on a 1/2^scale-size sample of every variant, one after another
    (generation excluded, as the reference times it)."""
    rels = rels or _cpu_rels(scale)
    results = [_cpu_join_timed(R, S, 0) for R, S in rels]
    secs = sum(r[0] for r in results)
    tuples = sum(len(R) + len(S) for R, S in rels)
    return {"value": tuples / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "oracle restatement of joins/CPU_JOIN/hash_cpu (partition by val %% 2^20 + bucket "
                      "nested loop, rows materialised into a preallocated array) on the three C3 variants at "
                      "1/%d size (R=2^%d, S=2^%d), one host thread, the variants one after another, "
                      "generation excluded" % (2 ** scale, 26 - scale, 28 - scale),
            "seconds": round(secs, 3), "rows": sum(r[1] for r in results)}


def run_reference(args) -> None:
    """Reference arm: the reference's multithreaded CPU hash join
    (joins/multi_joins/hash, restated; the reference's own binaries cannot be
    built where the reference sources are absent) with every host core, on a
    bounded 1/16-size sample of the three C3 variants per step."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    scale = 4
    nt = os.cpu_count() or 8
    rels = _cpu_rels(scale)

    def step():
        return sum(_cpu_join_timed(R, S, nt)[0] for R, S in rels)

    for _ in range(args.warmup):
        step()
    secs = [step() for _ in range(args.steps)]
    total_tuples = sum(len(R) + len(S) for R, S in rels)
    value = total_tuples * len(secs) / sum(secs)
    sample = ("oracle restatement of joins/multi_joins/hash (pthreads: partition by val %% 2^17 with per-thread "
              "counts and scatter, partitions claimed by threads and nested-looped, rows materialised into a "
              "preallocated array) on the three C3 variants at 1/%d size (R=2^%d, S=2^%d), %d threads, "
              "generation excluded" % (2 ** scale, 26 - scale, 28 - scale, nt))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": {"workload": WORKLOAD + " (CPU sample at 1/%d size)" % 2 ** scale},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_profile_case(name: str, scale: int, repeat: int) -> None:
    """A small case for profilers: `repeat` hash joins of one workload at
    1/2^scale size, each synchronised; prints the phase times of the last.
    d2 / d3: `repeat` distance joins of 2^(19 - scale) x 2^(19 - scale) points
    (after one count-only call); c5_batch: `repeat` batches of the served
    stream's 256 request instances; c4_index: `repeat` times a hash index and a
    sort index built on C4's R and probed with its S; c4_star: `repeat` star
    joins."""
    import torch

    from eating_one_gb300.build import build
    from eating_one_gb300.engine import Engine
    from eating_one_gb300.workloads import workload

    build()
    eng = Engine(0)
    if name == "c5_batch":  # the served stream's 256 request instances as one batch per call
        from eating_one_gb300 import native
        from eating_one_gb300.serve import RequestPool

        pool = RequestPool(eng, 256)
        descs = (native.JoinDesc * len(pool.desc))(*pool.desc)
        d_counts = torch.zeros(len(pool.desc), dtype=torch.int64, device="cuda")
        one_count = torch.zeros(1, dtype=torch.int64, device="cuda")
        stream = torch.cuda.current_stream()
        eng.batch_hash_join_async(descs, len(pool.desc), d_counts)  # warm-up: the arena grows once
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        for _ in range(repeat):
            eng.batch_hash_join_async(descs, len(pool.desc), d_counts)
        e1.record(stream)
        # the same joins one pipeline each, on the same stream
        for R, S, o in zip(pool.R, pool.S, pool.out):
            eng.hash_join_async(R, S, o, one_count)
        e2.record(stream)
        torch.cuda.synchronize()
        got = d_counts.cpu().tolist()
        assert got == pool.expected
        tuples = sum(pool.tuples(i) for i in range(len(pool.desc)))
        print(json.dumps({"profile_case": name, "joins": len(got), "rows": int(sum(got)), "tuples": tuples,
                          "batch_ms": round(e0.elapsed_time(e1) / repeat, 4),
                          "per_join_ms": round(e1.elapsed_time(e2), 4)}), flush=True)
        return
    if name == "c4_star":  # `repeat` 3-way star joins of C4's fact and dimension tables
        w = workload("c4_star", scale)
        t = {k: eng.generate(v) for k, v in w.items()}
        out = None
        for _ in range(repeat):
            out = eng.star_join3(t["F1"], t["F2"], t["D1"], t["D2"], out=out)
        print(json.dumps({"profile_case": name, "scale": scale, "F": int(t["F1"].shape[0]),
                          "rows": int(out.shape[0])}), flush=True)
        return
    if name == "c4_index":  # per repeat: a hash index and a sort index built on C4's R, each probed once
        w = workload("c4", scale)
        R, S = eng.generate(w["R"]), eng.generate(w["S"])
        n_out = eng.count("hash", R, S)
        out = torch.empty((n_out, 4), dtype=torch.int32, device="cuda")
        for _ in range(repeat):
            for kind in ("hash", "sort"):
                ix = eng.build_index(kind, R)
                try:
                    assert ix.join(S, out=out).shape[0] == n_out
                finally:
                    ix.free()
        print(json.dumps({"profile_case": name, "scale": scale, "R": int(R.shape[0]), "S": int(S.shape[0]),
                          "rows": n_out}), flush=True)
        return
    if name == "c3_build":  # `repeat` hash tables built on C3's R (the join's build phase alone)
        w = workload("c3_s1.0", scale)
        R = eng.generate(w["R"])
        for _ in range(repeat):
            eng.build_index("hash", R).free()
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "scale": scale, "R": int(R.shape[0])}), flush=True)
        return
    if name in ("d2", "d3"):  # distance joins: dist_screen_kernel x2 + dist_kernel per call
        from eating_one_gb300.native import point_result_dtype
        from eating_one_gb300.workloads import distance_workload

        dims, Rp, Sp = distance_workload(name, scale)
        dR, dS = eng.points_to_device(Rp), eng.points_to_device(Sp)
        n_out = eng.distance_join_count(dR, dS, dims)
        out = torch.empty((n_out, point_result_dtype(dims).itemsize), dtype=torch.uint8, device="cuda")
        for _ in range(repeat):
            assert eng.distance_join(dR, dS, dims, 1.0, out=out).shape[0] == n_out
        print(json.dumps({"profile_case": name, "scale": scale, "R": len(Rp), "S": len(Sp), "rows": n_out}),
              flush=True)
        return
    w = workload(name, scale)
    R, S = eng.generate(w["R"]), eng.generate(w["S"])
    n_out = eng.count("hash", R, S)
    out = torch.empty((n_out, 4), dtype=torch.int32, device="cuda")
    eng.set_timing(True)
    for _ in range(repeat):
        got = eng.hash_join(R, S, out=out)
        assert got.shape[0] == n_out
    print(json.dumps({"profile_case": name, "scale": scale, "R": int(R.shape[0]), "S": int(S.shape[0]),
                      "rows": n_out, "phases_ms": [round(x, 4) for x in eng.phase_ms()]}), flush=True)


SERVE_SWEEP = (0.25, 0.5, 0.75, 1.0, 1.25, 1.5, 1.75, 2.0, 2.25, 2.5, 2.75, 3.0)
SERVE_REPEATS = 3
SERVE_SLOS_MS = (2.0, 5.0, 10.0, 20.0)


def run_serve(n_requests: int, n_instances: int, lanes: int) -> None:
    """Configuration C5: the served request stream, batched vs one pipeline per join.

    Both modes first run the whole stream submitted at once (saturation), then
    Poisson arrivals at SERVE_SWEEP times the per-join saturation rate, each
    rate SERVE_REPEATS times (the run with the median p99 stands for it: a
    single run's p99 moves with a host stall).  For each p99 objective in
    SERVE_SLOS_MS, a mode's throughput is the highest achieved input-tuple rate
    among its rates whose p99 latency meets the objective; the batched/per-join
    ratio of those throughputs is the throughput at equal p99.  Each server is
    first warmed up by every instance, four times over, submitted at once, so
    that no lane's scratch grows inside a timed run."""
    import torch

    from eating_one_gb300.build import build
    from eating_one_gb300.engine import Engine
    from eating_one_gb300.serve import BATCHED, PER_JOIN, RequestPool, Server, run_stream

    build()
    eng = Engine(0)
    # every result is checked by its checksum (computed by the server on the
    # device) against the instance's result alone; lanes x 1024 requests can be
    # in flight, so each instance gets enough output buffers that no two of
    # them write to the same one
    copies = max(1, (lanes * 1024 + n_instances - 1) // n_instances)
    pool = RequestPool(eng, n_instances, copies=copies, checksums=True)
    modes = {"batched": BATCHED, "per_join": PER_JOIN}
    res = {m: {} for m in modes}
    warm = 4 * n_instances
    for name, mode in modes.items():
        srv = Server(mode, lanes=lanes, checksums=True)
        run_stream(srv, pool, warm, None, seed=7)  # warm-up: arenas grow once
        res[name]["saturation"] = run_stream(srv, pool, n_requests, None, seed=8)
        srv.close()
    base_rate = res["per_join"]["saturation"]["requests_per_s"]

    def median_run(runs):
        return sorted(runs, key=lambda r: r["p99_ms"])[len(runs) // 2]

    for name, mode in modes.items():
        srv = Server(mode, lanes=lanes, checksums=True)
        run_stream(srv, pool, warm, None, seed=7)
        res[name]["poisson"] = []
        for i, f in enumerate(SERVE_SWEEP):
            runs = [run_stream(srv, pool, n_requests, f * base_rate, seed=10 + 100 * k + i)
                    for k in range(SERVE_REPEATS)]
            r = median_run(runs)
            r["p99_ms_repeats"] = [x["p99_ms"] for x in runs]
            r["wrong"] = sum(x["wrong"] for x in runs)  # every repeat's results are checked
            res[name]["poisson"].append(r)
        srv.close()

    def best(name, slo):
        runs = res[name]["poisson"] + [res[name]["saturation"]]
        ok = [r["tuples_per_s"] for r in runs if r["p99_ms"] <= slo]
        return max(ok, default=0.0)

    at_slo = []
    for slo in SERVE_SLOS_MS:
        b, p = best("batched", slo), best("per_join", slo)
        at_slo.append({"p99_slo_ms": slo, "batched_tuples_per_s": b, "per_join_tuples_per_s": p,
                       "ratio": (b / p) if p > 0 else None})
    wrong = sum(r["wrong"] for m in res.values() for r in [m["saturation"]] + m["poisson"])
    line = {"workload": "C5 served stream: %d requests, |R| log-uniform in [2^10, 2^22], |S| = 4|R|, u in {1,2,8}, "
                        "Poisson arrivals; %d device-resident request instances" % (n_requests, n_instances),
            "lanes": lanes, "per_join_saturation_requests_per_s": base_rate, "sweep_factors": list(SERVE_SWEEP),
            "throughput_at_equal_p99": at_slo, "results": res,
            "saturation_ratio": res["batched"]["saturation"]["tuples_per_s"] /
                                res["per_join"]["saturation"]["tuples_per_s"],
            "wrong_results": wrong,
            "checked": "every result: count and the order-independent checksum of its rows (computed on the device "
                       "by the server) against the same join run alone"}
    print(json.dumps(line), flush=True)
    del torch


def config_lines(eng, peaks: dict, steps: int, distance: bool) -> list[dict]:
    """The other configurations, each timed with CUDA events over `steps`
    device-resident runs after warm-up: C1, C2, the C4 index, outer and star
    joins and (distance) the 2-D/3-D distance joins; one dict per configuration."""
    import torch

    from eating_one_gb300.workloads import workload

    props = torch.cuda.get_device_properties(0)
    stream = torch.cuda.current_stream()

    def timed(fn, n=steps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    def hbm(alg, ms):
        gbs = alg / (ms / 1000.0) / 1e9
        return {"alg_bytes": int(alg), "achieved_gbs": round(gbs, 1), "frac": round(gbs / peaks["hbm_gbs"], 4),
                "peak_source": peaks["source"]}

    lines = []
    # C1: the parity configuration at full size (count sizes the output, then the join writes it)
    w = workload("c1")
    R, S = eng.generate(w["R"]), eng.generate(w["S"])
    n = eng.count("hash", R, S)
    ms = timed(lambda: eng.hash_join(R, S))
    lines.append({"config": "C1 hash join R=2^20 unique x S=2^22 (count, then write)", "ms": round(ms, 4),
                  "rows": n, "tuples_per_s": (R.shape[0] + S.shape[0]) / (ms / 1000),
                  "roofline": hbm(24 * (R.shape[0] + S.shape[0]) + 16 * n, ms)})
    # C2: block nested loop, all 2^36 pairs
    w = workload("c2")
    R, S = eng.generate(w["R"]), eng.generate(w["S"])
    n = eng.count("bnl", R, S)
    out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    ms = timed(lambda: eng.join("bnl", R, S, out=out), max(3, steps // 4))
    pairs = R.shape[0] * S.shape[0]
    issue = props.multi_processor_count * 128 * 2.07e9  # one INT32 lane-instruction per clock per lane
    lines.append({"config": "C2 BNLJ R=2^16 x S=2^20, keys uniform in [0, 2^16)", "ms": round(ms, 4), "rows": n,
                  "pair_compares_per_s": pairs / (ms / 1000),
                  "roofline": {"bound": "int32 issue", "peak_lane_ops_per_s": issue,
                               "frac_at_one_op_per_compare": round(pairs / (ms / 1000) / issue, 4)},
                  "reference_gpu_log": "2^20 x 2^16 in 1.483 s (nestLoopJoin, sm_35)"})
    del out
    # C4: index joins, outer join, star join
    w = workload("c4")
    R, S = eng.generate(w["R"]), eng.generate(w["S"])
    for kind in ("hash", "sort"):
        t_build = timed(lambda: eng.build_index(kind, R).free(), 3)
        ix = eng.build_index(kind, R)
        n = ix.count(S)
        out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        ms = timed(lambda: ix.join(S, out=out))
        lines.append({"config": "C4 %s-index join R=2^24 x S=2^26 (50%% match)" % kind, "probe_ms": round(ms, 4),
                      "build_ms": round(t_build, 4), "rows": n,
                      "tuples_per_s": (R.shape[0] + S.shape[0]) / ((ms + t_build) / 1000),
                      "roofline": hbm(16 * R.shape[0] + 8 * S.shape[0] + 16 * n, ms + t_build)})
        ix.free()
    n = eng.count("left_outer", R, S)
    out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    ms = timed(lambda: eng.join("left_outer", R, S, out=out))
    lines.append({"config": "C4 left outer join R=2^24 x S=2^26", "ms": round(ms, 4), "rows": n,
                  "tuples_per_s": (R.shape[0] + S.shape[0]) / (ms / 1000),
                  "roofline": hbm(24 * (R.shape[0] + S.shape[0]) + 16 * n, ms)})
    del out
    w = workload("c4_star")
    t = {k: eng.generate(v) for k, v in w.items()}
    args = (t["F1"], t["F2"], t["D1"], t["D2"])
    n = eng.star_join3(*args).shape[0]
    out = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    ms = timed(lambda: eng.star_join3(*args, out=out))
    nd = t["D1"].shape[0] + t["D2"].shape[0]
    lines.append({"config": "C4 star join F=2^26 x D1, D2 = 2^20", "ms": round(ms, 4), "rows": n,
                  "tuples_per_s": (2 * t["F1"].shape[0] + nd) / (ms / 1000),
                  "roofline": hbm(8 * nd + 16 * t["F1"].shape[0] + 32 * n, ms)})
    del out, t
    if not distance:
        return lines
    # distance joins: all 2^38 pairs of 2^19 x 2^19 reference-shaped points, radius 1
    from eating_one_gb300.native import point_result_dtype
    from eating_one_gb300.workloads import distance_workload
    from oracle import oracle as O

    fp32 = props.multi_processor_count * 128 * 2.07e9  # one FP32 lane-instruction per clock per lane
    for name in ("d2", "d3"):
        dims, Rp, Sp = distance_workload(name)
        dR, dS = eng.points_to_device(Rp), eng.points_to_device(Sp)
        n = eng.distance_join_count(dR, dS, dims)
        out = torch.empty((n, point_result_dtype(dims).itemsize), dtype=torch.uint8, device="cuda")
        ms = timed(lambda: eng.distance_join(dR, dS, dims, 1.0, out=out), max(3, steps // 4))
        pairs = len(Rp) * len(Sp)
        # CPU: the oracle restatement on every host core, over a bounded slice of S
        threads = os.cpu_count() or 1
        s_sample = Sp[:1024]
        t0 = time.perf_counter()
        O.distance_join(dims, Rp, s_sample, 1.0, threads=threads)
        cpu_s = time.perf_counter() - t0
        lines.append({"config": "%dD distance join R=2^19 x S=2^19 points, radius 1, 10%% copies" % dims,
                      "ms": round(ms, 4), "rows": n, "pairs_per_s": pairs / (ms / 1000),
                      "roofline": {"bound": "fp32 issue", "peak_lane_ops_per_s": fp32,
                                   "frac_at_two_ops_per_pair": round(2 * pairs / (ms / 1000) / fp32, 4)},
                      "cpu_baseline": {"pairs_per_s": len(Rp) * len(s_sample) / cpu_s, "cores": threads,
                                       "kind": "port", "sample": "R=2^19 x the first 1024 S points"},
                      "reference_cpu_log": "2-D 2^19 x 2^19 in 3718 s (complex_block/2d_cpu/nohup.out)"})
    return lines


def run_configs(steps: int) -> None:
    """`--configs`: every other configuration, one JSON line each, distance joins included."""
    from eating_one_gb300.build import build
    from eating_one_gb300.engine import Engine

    build()
    eng = Engine(0)
    for ln in config_lines(eng, load_peaks(), steps, distance=True):
        print(json.dumps(ln), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="leave out the C1, C2 and C4 timings")
    ap.add_argument("--profile", default=None, help="run a small profiling case of this workload instead")
    ap.add_argument("--scale", type=int, default=3)
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--serve", action="store_true", help="run the served-stream sweep (configuration C5)")
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--lanes", type=int, default=2)
    ap.add_argument("--configs", action="store_true", help="time configurations C1, C2, C4 and the 2-D/3-D distance joins instead")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.configs:
        run_configs(args.steps if args.steps != 30 else 10)
        return
    if args.serve:
        run_serve(args.requests, args.instances, args.lanes)
        return
    if args.profile:
        run_profile_case(args.profile, args.scale, args.repeat)
        return
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    from eating_one_gb300.build import build
    from eating_one_gb300.engine import Engine
    from eating_one_gb300.workloads import alg_bytes, workload

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if rank == 0:
        build()
    if dist:
        dist.barrier()
    eng = Engine(local)
    peaks = load_peaks()

    # inputs (weak scaling: every rank joins its own seeded relations)
    joins = []
    for v in VARIANTS:
        w = workload(v)
        for side in ("R", "S"):
            w[side].seed ^= (rank * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        R, S = eng.generate(w["R"]), eng.generate(w["S"])
        joins.append({"name": v, "R": R, "S": S, "out": None, "n_out": None})
    units = sum(j["R"].shape[0] + j["S"].shape[0] for j in joins)

    def step():
        # the reference's sequence per join (hj.cc:997-1115): the count pass,
        # the count read back to the host, an output of exactly that size, the
        # write (which reuses the count's table, partitioned S and run
        # descriptors); the previous step's output is released first, so the
        # caching allocator hands the same memory back
        for j in joins:
            j["out"] = None
            n = eng.count("hash", j["R"], j["S"])
            j["out"] = torch.empty((n, 4), dtype=torch.int32, device="cuda")
            j["n_out"] = n
            eng.hash_join(j["R"], j["S"], out=j["out"])

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    assert eng.sync_status() == 0, eng.last_error()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    eng.set_timing(True)
    eng.phase_totals()
    launches0 = eng.kernel_launches()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = eng.kernel_launches() - launches0
    phases, _ = eng.phase_totals()
    eng.set_timing(False)
    ms = e0.elapsed_time(e1) / args.steps

    # every join's rows against the oracle's full-size digest (count and
    # order-independent checksum, tests/golden/fullsize.json); other ranks'
    # relations are seeded differently, so there only the count is checked
    # against the join's own count pass
    status = eng.sync_status()
    assert status == 0, "device status %d: %s" % (status, eng.last_error())
    parity = {}
    gold = {}
    gpath = os.path.join(ROOT, "tests", "golden", "fullsize.json")
    if rank == 0 and os.path.exists(gpath):
        with open(gpath) as f:
            gold = json.load(f)
    for j in joins:
        got = {"count": int(j["out"].shape[0]), "checksum": eng.checksum(j["out"])}
        want = gold.get(j["name"], {}).get("inner")
        if want is not None:
            assert got == want, (j["name"], got, want)
            parity[j["name"]] = "count %d and checksum %d equal to the oracle's" % (got["count"], got["checksum"])

    per_rank = gather_ms(ms, dist, torch.device("cuda", local))
    value, ms_max = aggregate(per_rank, units, 1)

    # roofline of the dominant phase (per join, averaged over the timed joins)
    nj = len(joins) * args.steps
    n_s = sum(j["S"].shape[0] for j in joins) / len(joins)
    n_r = sum(j["R"].shape[0] for j in joins) / len(joins)
    n_o = sum(j["n_out"] for j in joins) / len(joins)
    names = ["build (R table: two MSD radix passes, a shared-memory sort per bucket group, key directory)",
             "partition (S radix pass)",
             "count (probe_count_dir_kernel: every probe's directory entry, stored as its run descriptor; "
             "scan of the warp-tile totals)",
             "write (probe_write_kernel: rows from the run descriptors at the scanned offsets)"]
    kernel = ["msd_local_kernel+rx_scatter_kernel+rx_hist_kernel (R)", "rx_scatter_kernel+rx_hist_kernel (S)",
              "probe_count_dir_kernel", "probe_write_kernel"]
    # algorithmic bytes per launch of each phase: the build reads R once and
    # writes its two columns (16 B per row), the partition reads and writes S
    # (16 B per tuple), the count reads the probe and writes its run
    # descriptor, the write reads the probe and its descriptor and writes the
    # rows (16 B per row); descriptors are 4 bytes for tables under 2^27 rows
    # (C3's 2^26), else 8
    desc = 4.0 if n_r < (1 << 27) else 8.0
    phase_bytes = [16.0 * n_r, 16.0 * n_s, (8.0 + desc) * n_s, (8.0 + desc) * n_s + 16.0 * n_o]
    per_join = [p / nj for p in phases]
    dom = max(range(4), key=lambda i: per_join[i])
    achieved = phase_bytes[dom] / (per_join[dom] / 1000.0) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_c3.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            traffic = json.load(f).get(kernel[dom])
    alg = sum(alg_bytes("hash", j["R"].shape[0], j["S"].shape[0], j["n_out"]) for j in joins)
    join_gbs = alg / (ms_max / 1000.0) / 1e9

    # the other configurations (C1, C2, C4), device-timed on the same GPU
    secondary = None
    if rank == 0 and not args.no_secondary:
        for j in joins:
            j["out"] = None
        torch.cuda.empty_cache()
        secondary = config_lines(eng, peaks, 10, distance=False)
    clk = clocks.stop()

    # end to end through the host-buffer C ABI call
    e2e = None
    if args.e2e_steps > 0:
        hosts = []
        for j in joins:
            j["out"] = None
        torch.cuda.empty_cache()
        max_out = max(j["n_out"] for j in joins)
        out_h = torch.empty((max_out, 4), dtype=torch.int32, pin_memory=True)
        for j in joins:
            hosts.append((j["R"].cpu().pin_memory(), j["S"].cpu().pin_memory(), j["n_out"]))
        eng.join_host_chunked("hash", hosts[0][0], hosts[0][1], out_h)  # warm-up
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            for Rh, Sh, n_out in hosts:
                n = eng.join_host_chunked("hash", Rh, Sh, out_h)
                assert n == n_out
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        link = link_bandwidth(out_h)
        if dist:
            t = torch.tensor([e2e_s], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = int(sum(8 * (R.shape[0] + S.shape[0]) for R, S, _ in hosts))
        d2h = int(sum(16 * n for _, _, n in hosts))
        e2e = {"value": units * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": round(e2e_s * 1000.0, 3),
               "api": "ej_join_host_chunked (pinned host R, S and out; 2^25-row S chunks, each chunk counted "
                      "before its rows are written)",
               "link": dict(link, floor_ms=round(1000.0 * max(h2d / (link["both_gbs"] * 1e9),
                                                               d2h / (link["both_gbs"] * 1e9)), 2))}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(4)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded device generators)",
        "config": {"workload": WORKLOAD, "R": 1 << 26, "S": 1 << 28, "joins_per_step": len(joins),
                   "results_per_step": int(sum(j["n_out"] for j in joins)),
                   "step": "per join: count pass (ej_hash_join_count: R table build, S partition, count "
                           "with run descriptors, scan), count read back, output of that size, write "
                           "(ej_hash_join, from the count's descriptors)",
                   "l2": "inputs larger than L2 (R 512 MB, S 2 GB per join)", "parallelism": "dp%d" % world},
        "parity": parity,
        "roofline": {"bound": "hbm", "kernel": kernel[dom], "phase": names[dom],
                     "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic,
                     "traffic_source": "not measured in this run: dram__bytes_read.sum + dram__bytes_write.sum "
                                       "of a 1/8-size ncu capture of the same kernel, scaled by 8 "
                                       "(profiles/traffic_c3.json, with the command that made it)",
                     "peak_source": peaks["source"],
                     "bytes_per_launch": int(phase_bytes[dom]), "ms_per_launch": round(per_join[dom], 4)},
        "join_roofline": {"alg_bytes_per_step": int(alg), "achieved": round(join_gbs, 1), "unit": "GB/s",
                          "frac": round(join_gbs / peaks["hbm_gbs"], 4), "peak_source": peaks["source"]},
        "phases_ms_per_join": {"build": round(per_join[0], 4), "partition": round(per_join[1], 4),
                               "count": round(per_join[2], 4), "write": round(per_join[3], 4)},
        "secondary": secondary,
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
