#!/usr/bin/env python3
"""Write tests/golden/fullsize.json: the oracle's result count and
order-independent checksum of every full-size join workload.

TEST INFRASTRUCTURE.  The results of the full-size workloads (up to 9.7e8
rows, 15.5 GB per join) do not fit the tests' host memory budget as rows, so
the oracle digests them instead: the relations are generated on the host with
the seeded generators of include/ej_gen.h (the same rows the device generators
give), and oracle/ej_oracle.c's ejo_join_digest_mt / ejo_star_digest_mt feed
every result row to the checksum that ej_checksum computes on the device.
The GPU tests (tests/test_fullsize_gpu.py) and bench.py compare the engine's
full-size results with these values.

    python tests/golden/make_fullsize.py [--threads N] [--only NAME ...]

Entries:
  c3_s0.0, c3_s0.75, c3_s1.0  inner join of R 2^26 (2^24 keys x4) and S 2^28
  c4                         inner join (hash and sort index) and left outer
                             join of R 2^24 and S 2^26
  c4_star                    3-way star join of F 2^26 with D1, D2 2^20
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "fullsize.json")
NAMES = ["c3_s0.0", "c3_s0.75", "c3_s1.0", "c4", "c4_star"]


def digest_entry(name: str, threads: int) -> dict:
    from eating_one_gb300.workloads import workload
    from oracle import oracle as O

    w = workload(name)
    if name == "c4_star":
        t = {k: O.generate(v, threads) for k, v in w.items()}
        n, c = O.star_digest(t["F1"], t["F2"], t["D1"], t["D2"], threads=threads)
        return {"F": int(w["F1"].n), "D1": int(w["D1"].n), "D2": int(w["D2"].n),
                "star": {"count": n, "checksum": c}}
    R, S = O.generate(w["R"], threads), O.generate(w["S"], threads)
    e = {"R": int(w["R"].n), "S": int(w["S"].n)}
    n, c = O.join_digest(R, S, threads=threads)
    e["inner"] = {"count": n, "checksum": c}
    if name == "c4":
        n, c = O.join_digest(R, S, outer=True, threads=threads)
        e["outer"] = {"count": n, "checksum": c}
    return e


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 8)
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    data["_about"] = ("oracle digests (count, order-independent checksum as ej_checksum) of the full-size "
                      "workloads of eating_one_gb300/workloads.py; made by tests/golden/make_fullsize.py")
    for name in args.only or NAMES:
        t0 = time.time()
        data[name] = digest_entry(name, args.threads)
        print(name, json.dumps(data[name]), "%.1f s" % (time.time() - t0), flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
