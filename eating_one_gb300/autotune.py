"""Autotuner: per size class of the build side, the hash join's knobs that
join fastest, chosen by timing candidates on the device:

  partition_bits  S radix bits (0 = probe in place, 1..8 = one radix pass of
                  that many bits; the probe side's "passes" is 0 or 1)
  bucket_delta    the table's load factor: about 4 * 2^-delta R rows per bucket
  build           the table build's radix passes: EJ_BUILD_LSD (four stable
                  8-bit passes of three launches each), EJ_BUILD_MSD (two
                  unordered 8-bit passes and a shared-memory sort per 16-bit
                  bucket) or EJ_BUILD_ONESWEEP (four stable 8-bit passes of
                  one launch each)
  table           how probes find runs: EJ_TABLE_FORMAT_BUCKETS (bucket
                  bounds) or EJ_TABLE_FORMAT_DIRECTORY (key directory)
  probe_warps     block shape of the probe kernels: 4 or 8 warps per block

The search is coordinate-wise from the planner's own choices (which are
timed first and stay a candidate of every knob), one knob at a time in the
order above, keeping each knob's fastest value.  The class's workload is the
served stream's request shape: |R| = 2^log2_rows unique keys, |S| = 4|R|
keys uniform over twice R's key range (half of S matches).

The reference tunes by hand: alternative #define sets per size class are
commented in its tuple.h files (joins/innerJoin_gpu/main_street/tuple.h:9-34,
joins/hashJoin_gpu/main_street/tuple.h:19-36).  Here the table is measured
and loaded into a handle with ej_set_tuning (TUNED_TABLE, measured on one
GB300, is what Engine loads by default); options set explicitly with
ej_set_option still win.

    python -m eating_one_gb300.autotune --out eating_one_gb300/tuning_gb300.json
"""
from __future__ import annotations

import argparse
import json
import os

import torch

from . import native
from .engine import Engine
from .workloads import EJ_GEN_PERM, EJ_GEN_UNIFORM, make_spec

TUNED_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")

PARTITION_CANDIDATES = (0, 4, 6, 7, 8)
DELTA_CANDIDATES = (-1, 0, 1)
BUILD_CANDIDATES = (native.EJ_BUILD_LSD, native.EJ_BUILD_MSD, native.EJ_BUILD_ONESWEEP)
TABLE_CANDIDATES = (native.EJ_TABLE_FORMAT_BUCKETS, native.EJ_TABLE_FORMAT_DIRECTORY)
WARPS_CANDIDATES = (4, 8)
KNOBS = ("partition_bits", "bucket_delta", "build", "table", "probe_warps")
PLANNER = {"partition_bits": -1, "bucket_delta": 0, "build": 0, "table": 0, "probe_warps": 0}
OPTION = {"partition_bits": "partition_bits", "bucket_delta": "bucket_bits_delta", "build": "build",
          "table": "table", "probe_warps": "probe_warps"}


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


def _apply(eng: Engine, cfg: dict) -> None:
    for k in KNOBS:
        eng.set_option(OPTION[k], cfg[k])


def class_workload(eng: Engine, log2_rows: int, seed: int = 77):
    nR = 1 << log2_rows
    R = eng.generate(make_spec(EJ_GEN_PERM, nR, 2 * nR, seed, seed + 1))
    S = eng.generate(make_spec(EJ_GEN_UNIFORM, 4 * nR, 2 * nR, seed + 2))
    return R, S


def time_config(eng: Engine, R, S, out, cfg: dict, reps: int) -> float:
    _apply(eng, cfg)
    try:
        return _time_join(eng, R, S, out, reps)
    finally:
        _apply(eng, PLANNER)


def tune_class(eng: Engine, log2_rows: int, reps: int = 3, seed: int = 77) -> dict:
    """The fastest knobs for the class's workload (see the module docstring)."""
    R, S = class_workload(eng, log2_rows, seed)
    out = torch.empty((eng.count("hash", R, S), 4), dtype=torch.int32, device=eng.device)
    candidates = {"partition_bits": [p for p in PARTITION_CANDIDATES if p <= max(log2_rows - 2, 0)],
                  "bucket_delta": list(DELTA_CANDIDATES), "build": list(BUILD_CANDIDATES),
                  "table": list(TABLE_CANDIDATES), "probe_warps": list(WARPS_CANDIDATES)}
    best = dict(PLANNER)
    best_ms = planner_ms = time_config(eng, R, S, out, best, reps)
    trials = [[round(planner_ms, 4), dict(best)]]
    for knob in KNOBS:
        for v in candidates[knob]:
            cfg = dict(best, **{knob: v})
            ms = time_config(eng, R, S, out, cfg, reps)
            trials.append([round(ms, 4), cfg])
            if ms < best_ms:
                best, best_ms = cfg, ms
    return dict(best, log2_rows=log2_rows, ms=round(best_ms, 4), planner_ms=round(planner_ms, 4), trials=trials)


def autotune(eng: Engine, classes=(10, 12, 14, 16, 18, 20, 22), reps: int = 3) -> list[dict]:
    """Tune every class; the engine's tuning table is cleared first (so that
    "planner" means the planner) and left empty.  The table ends with an
    entry one class above the last that hands every larger build side back to
    the planner: the classes' workload is the served stream's request shape,
    and beyond its sizes (2^22 rows) the right table format depends on the
    data (the planner keeps a key directory when the table's runs average two
    rows or more), which no single workload stands for."""
    load(eng, [])
    table = [tune_class(eng, c, reps) for c in classes]
    if table:
        table.append(dict(PLANNER, log2_rows=max(classes) + 1, ms=None, planner_ms=None, trials=[]))
    return table


def load(eng: Engine, table: list[dict]) -> None:
    """Install a tuning table (autotune() result or its JSON) into the engine's handle."""
    arr = (native.TuneEntry * max(len(table), 1))()
    for i, e in enumerate(table):
        arr[i].log2_rows = e["log2_rows"]
        arr[i].partition_bits = e.get("partition_bits", -1)
        arr[i].bucket_delta = e.get("bucket_delta", 0)
        arr[i].build = e.get("build", 0)
        arr[i].table = e.get("table", 0)
        arr[i].probe_warps = e.get("probe_warps", 0)
    eng._check(eng.lib.ej_set_tuning(eng.h, arr, len(table)))


def load_default(eng: Engine) -> bool:
    """Install TUNED_TABLE when it exists; True when a table was installed."""
    if not os.path.exists(TUNED_TABLE):
        return False
    with open(TUNED_TABLE) as f:
        load(eng, json.load(f)["table"])
    return True


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--classes", default="10,12,14,16,18,20,22")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    eng = Engine(0, tuned=False)
    table = autotune(eng, tuple(int(x) for x in args.classes.split(",")), args.reps)
    doc = {"about": "hash-join knobs per build-side size class, measured on one GB300 by "
                    "eating_one_gb300/autotune.py (best of %d timed joins per candidate)" % args.reps,
           "device": torch.cuda.get_device_name(0), "table": table}
    text = json.dumps(doc, indent=1)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text + "\n")
    print(text)


if __name__ == "__main__":
    main()
