"""Autotuner: per size class of the build side, pick the S partition bits
(0 = probe in place, 1..8 = one radix pass of that many bits; "passes" is
0 or 1) and the bucket-bits delta (the table's load factor: about 4 * 2^-delta
R rows per bucket) that join fastest, by timing candidates on the device.

The reference tunes by hand: alternative #define sets per size class are
commented in its tuple.h files (joins/innerJoin_gpu/main_street/tuple.h:9-34,
joins/hashJoin_gpu/main_street/tuple.h:19-36).  Here the table is measured
and loaded into a handle with ej_set_tuning; options set explicitly with
ej_set_option still win.

    python -m eating_one_gb300.autotune --out tuning.json [--classes 10,14,18,22,26]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import torch

from . import native
from .engine import Engine
from .workloads import EJ_GEN_PERM, EJ_GEN_UNIFORM, make_spec

PARTITION_CANDIDATES = (0, 4, 6, 8)
DELTA_CANDIDATES = (-1, 0, 1)


def _time_join(eng: Engine, R, S, out, reps: int) -> float:
    stream = torch.cuda.current_stream()
    eng.hash_join(R, S, out=out)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.hash_join(R, S, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune_class(eng: Engine, log2_rows: int, reps: int = 3, seed: int = 77) -> dict:
    """Best (partition_bits, bucket_delta) for |R| = 2^log2_rows unique keys and
    |S| = 4|R| keys uniform over twice R's key range (half of S matches)."""
    nR = 1 << log2_rows
    R = eng.generate(make_spec(EJ_GEN_PERM, nR, 2 * nR, seed, seed + 1))
    S = eng.generate(make_spec(EJ_GEN_UNIFORM, 4 * nR, 2 * nR, seed + 2))
    out = torch.empty((eng.count("hash", R, S), 4), dtype=torch.int32, device=eng.device)
    trials = []
    for pb in PARTITION_CANDIDATES:
        if pb > max(log2_rows - 2, 0):
            continue
        for delta in DELTA_CANDIDATES:
            eng.set_option("partition_bits", pb)
            eng.set_option("bucket_bits_delta", delta)
            trials.append((_time_join(eng, R, S, out, reps), pb, delta))
    eng.set_option("partition_bits", -1)
    eng.set_option("bucket_bits_delta", 0)
    planner = _time_join(eng, R, S, out, reps)
    ms, pb, delta = min(trials)
    return {"log2_rows": log2_rows, "partition_bits": pb, "bucket_delta": delta, "ms": round(ms, 4),
            "planner_ms": round(planner, 4), "trials": [[round(t, 4), p, d] for t, p, d in trials]}


def autotune(eng: Engine, classes=(10, 12, 14, 16, 18, 20, 22, 24, 26), reps: int = 3) -> list[dict]:
    return [tune_class(eng, c, reps) for c in classes]


def load(eng: Engine, table: list[dict]) -> None:
    """Install a tuning table (autotune() result or its JSON) into the engine's handle."""
    arr = (native.TuneEntry * max(len(table), 1))()
    for i, e in enumerate(table):
        arr[i].log2_rows, arr[i].partition_bits = e["log2_rows"], e["partition_bits"]
        arr[i].bucket_delta, arr[i].reserved = e["bucket_delta"], 0
    eng._check(eng.lib.ej_set_tuning(eng.h, arr, len(table)))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--classes", default="10,12,14,16,18,20,22,24,26")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    eng = Engine(0)
    table = autotune(eng, tuple(int(x) for x in args.classes.split(",")), args.reps)
    text = json.dumps(table)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text)
    del C


if __name__ == "__main__":
    main()
