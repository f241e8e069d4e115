"""Golden fixtures: loaders for the reference's join_ori tables and recorded reference runs."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def join_ori():
    """The reference's known-answer tables joins/join_ori/R and S as (n, 2) int32 arrays."""
    z = np.load(os.path.join(HERE, "join_ori.npz"))
    out = []
    for v in (z["R_val"], z["S_val"]):
        t = np.empty((len(v), 2), dtype=np.int32)
        t[:, 0] = np.arange(len(v))
        t[:, 1] = v
        out.append(t)
    return out[0], out[1]


def reference_runs():
    with open(os.path.join(HERE, "reference_runs.json")) as f:
        return json.load(f)
