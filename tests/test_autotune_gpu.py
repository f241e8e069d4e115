"""The autotuner: every knob it sets gives the oracle's rows, it measures
candidates per size class, and the committed table it measured on GB300
(eating_one_gb300/tuning_gb300.json, loaded by Engine by default) is never
slower than the planner on the class it was tuned for."""
import json
import os

import numpy as np
import pytest
import torch

from eating_one_gb300 import autotune, native
from eating_one_gb300.workloads import workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


@pytest.mark.parametrize("build", [native.EJ_BUILD_LSD, native.EJ_BUILD_MSD, native.EJ_BUILD_ONESWEEP])
@pytest.mark.parametrize("table", [native.EJ_TABLE_FORMAT_BUCKETS, native.EJ_TABLE_FORMAT_DIRECTORY])
@pytest.mark.parametrize("warps", [4, 8])
def test_every_knob_gives_the_oracle_rows(engine, build, table, warps):
    rng = np.random.default_rng(build * 10 + table * 3 + warps)
    R = np.stack([np.arange(30011), rng.integers(-2000, 9000, 30011)], 1).astype(np.int32)
    S = np.stack([np.arange(30011, 130011), rng.integers(-2500, 9500, 100000)], 1).astype(np.int32)
    R[:300, 1] = 77  # one long run
    S[:5, 1] = 77
    for name, v in (("build", build), ("table", table), ("probe_warps", warps), ("partition_bits", 5)):
        engine.set_option(name, v)
    try:
        got = {a: engine.join(a, dev(R), dev(S))
               for a in ("hash", "single_hash", "left_outer", "hash_index", "sort_index")}
        out = torch.empty((len(O.hash_join(R, S)), 4), dtype=torch.int32, device="cuda")
        got["one_pass"] = engine.hash_join(dev(R), dev(S), out=out)  # no count before it
    finally:
        for name, v in (("build", 0), ("table", 0), ("probe_warps", 0), ("partition_bits", -1)):
            engine.set_option(name, v)
    inner, outer = O.canon(O.hash_join(R, S)), O.canon(O.left_outer_join(R, S))
    for a, rows in got.items():
        assert np.array_equal(O.canon(rows.cpu().numpy()), outer if a == "left_outer" else inner), a


def test_autotune_small_classes(engine):
    table = autotune.autotune(engine, classes=(10, 14), reps=1)
    assert [e["log2_rows"] for e in table] == [10, 14, 15]
    assert all(table[-1][k] == v for k, v in autotune.PLANNER.items())  # larger tables: the planner
    for e in table[:-1]:
        assert e["partition_bits"] in (-1,) + autotune.PARTITION_CANDIDATES
        assert e["bucket_delta"] in autotune.DELTA_CANDIDATES
        assert e["build"] in (0,) + autotune.BUILD_CANDIDATES
        assert e["ms"] <= min(t[0] for t in e["trials"]) + 1e-9 and e["ms"] <= e["planner_ms"]
    # an extreme table: S partitioned with 8 bits, small buckets, LSD, a
    # directory and 4-warp blocks everywhere
    autotune.load(engine, [{"log2_rows": 0, "partition_bits": 8, "bucket_delta": 1, "build": 1, "table": 2,
                            "probe_warps": 4}])
    try:
        w = workload("c3_s0.75", scale=8)
        R, S = O.generate(w["R"]), O.generate(w["S"])
        got = engine.hash_join(engine.generate(w["R"]), engine.generate(w["S"]))
        assert np.array_equal(O.canon(got.cpu().numpy()), O.canon(O.hash_join(R, S)))
    finally:
        autotune.load_default(engine) or autotune.load(engine, [])


def test_tuned_table_not_slower_than_planner(engine):
    """Re-measured here: for each class of the committed table up to 2^22 rows,
    the tuned knobs join at least as fast as the planner's (best of 5 joins
    each; 5% + 20 us allowed for timing noise)."""
    assert os.path.exists(autotune.TUNED_TABLE)
    with open(autotune.TUNED_TABLE) as f:
        table = json.load(f)["table"]
    autotune.load(engine, [])  # the planner alone, and the tuned knobs as options
    try:
        for e in table:
            if e["log2_rows"] > 22:
                continue
            R, S = autotune.class_workload(engine, e["log2_rows"])
            out = torch.empty((engine.count("hash", R, S), 4), dtype=torch.int32, device="cuda")
            tuned = autotune.time_config(engine, R, S, out, {k: e[k] for k in autotune.KNOBS}, 5)
            planner = autotune.time_config(engine, R, S, out, autotune.PLANNER, 5)
            assert tuned <= planner * 1.05 + 0.02, (e["log2_rows"], tuned, planner)
    finally:
        autotune.load_default(engine)
