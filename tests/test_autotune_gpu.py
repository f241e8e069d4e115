"""The autotuner measures candidates per size class and installs a table that
the planner follows; joins stay bit-exact under any table."""
import numpy as np
import pytest

from eating_one_gb300 import autotune
from eating_one_gb300.workloads import workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_autotune_small_classes(engine):
    table = autotune.autotune(engine, classes=(10, 14), reps=1)
    assert [e["log2_rows"] for e in table] == [10, 14]
    for e in table:
        assert e["partition_bits"] in autotune.PARTITION_CANDIDATES
        assert e["bucket_delta"] in autotune.DELTA_CANDIDATES
        assert e["ms"] <= min(t[0] for t in e["trials"]) + 1e-9
    # an extreme table: partition S with 8 bits and small buckets everywhere
    autotune.load(engine, [{"log2_rows": 0, "partition_bits": 8, "bucket_delta": 1}])
    try:
        w = workload("c3_s0.75", scale=8)
        R, S = O.generate(w["R"]), O.generate(w["S"])
        got = engine.hash_join(engine.generate(w["R"]), engine.generate(w["S"]))
        assert np.array_equal(O.canon(got.cpu().numpy()), O.canon(O.hash_join(R, S)))
    finally:
        autotune.load(engine, [])
