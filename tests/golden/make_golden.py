"""Generate the golden fixtures that pin the oracle to the reference's own output.

Run with $EJ_REFERENCE naming the reference checkout; the GPU tests and the
bench never run this script.

1. join_ori known-answer fixture: the reference's binary tables
   joins/join_ori/R (1000 tuples) and S (100000 tuples) are stored compressed
   in join_ori.npz, and the four reference programs that join them
   (joins/join_ori/{bnlj,hj,inner-idx-bnlj,outer-idx-bnlj}.cc, built from
   source by oracle/build_ref.sh) are run on them; their printed
   `resultVal` (sum of rval over all matches) goes to reference_runs.json.
2. CPU_JOIN runs: the unmodified joins/CPU_JOIN/{hash_cpu,inner_cpu,
   sortIndex_cpu,block_cpu} programs are fed seeded relations through
   oracle/ref_shim.cpp; the match count each prints and, where the program
   materialises rows, the order-independent checksum of those rows (mapped to
   RESULT{rkey, rval, lkey, lval} with r = right/R) are recorded.
3. Distance joins: the unmodified joins/CPU_JOIN/3d_cpu and
   joins/blockJoin_gpu/complex_block/2d_cpu programs (radius DISTANCE = 1) are
   fed points the same way: reference-shaped inputs (integer values, 10%
   copies) and boundary cases (tests.golden.boundary_points).  The inputs go
   to distance.npz, the printed count and the sha256 of the canonical rows
   (oracle.point_rows_digest) to reference_runs.json["distance"].

`--distance-only` redoes part 3 alone and keeps the rest of reference_runs.json.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from eating_one_gb300.workloads import distance_points, workload  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden import boundary_points  # noqa: E402

REF = os.environ.get("EJ_REFERENCE", "")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")

# (program, workload, scale): R keys 1..|R|, S keys |R|+1..|R|+|S| as the
# reference's shared getTupleId() counter numbers them
CASES = [
    ("hash_cpu", "c1", 4),
    ("hash_cpu", "c3_s1.0", 8),
    ("inner_cpu", "c1", 4),
    ("inner_cpu", "c3_s0.75", 8),
    ("sortindex_cpu", "c1", 4),
    ("sortindex_cpu", "c3_s0.0", 8),
    ("block_cpu", "c2", 4),
]

# how each program lays out its 16-byte result rows -> our (rkey, rval, lkey, lval)
ROW_MAP = {
    "inner_cpu": [2, 3, 0, 1],      # {rkey=lt.key, rval=lt.val, skey=rt.key, sval=rt.val}
    "sortindex_cpu": [0, 1, 2, 3],  # {rkey=rt.key, rval, lkey=lt.key, lval}
    "block_cpu": [3, 1, 2, 0],      # JOIN_TUPLE {lval, rval, lid, rid}
}


def relations(name: str, scale: int):
    w = workload(name, scale)
    w["R"].key_base = 1
    w["S"].key_base = 1 + w["R"].n
    return O.generate(w["R"]), O.generate(w["S"]), w


def write_table(path: str, t: np.ndarray) -> None:
    with open(path, "wb") as f:
        np.array([len(t)], dtype=np.int32).tofile(f)
        np.ascontiguousarray(t, dtype=np.int32).tofile(f)


def run_cpu_join(prog: str, R: np.ndarray, S: np.ndarray):
    with tempfile.TemporaryDirectory() as tmp:
        rp, sp, dp = (os.path.join(tmp, x) for x in ("R.tbl", "S.tbl", "rows.bin"))
        write_table(rp, R)
        write_table(sp, S)
        out = subprocess.run([os.path.join(REF_BIN, prog), rp, sp, dp], cwd=tmp, check=True,
                             stdout=subprocess.PIPE, text=True).stdout
        if prog == "block_cpu":
            count = int(re.findall(r"^(\d+)$", out, re.M)[0])
        else:
            count = int(re.findall(r"resultVal: (\d+)", out)[0])
        rows = None
        if os.path.exists(dp):
            rows = np.fromfile(dp, dtype=np.int32).reshape(-1, 4)[:, ROW_MAP[prog]]
        diffs = [int(x) for x in re.findall(r"Diff: (\d+) us", out)]
        return count, rows, diffs, out


# (case, dims, generator): radius 1, the reference programs' DISTANCE
DIST_CASES = [
    ("ref_shape_2d", 2, lambda: distance_points(2, 1000, 1500, 0xD157_0002)),
    ("ref_shape_3d", 3, lambda: distance_points(3, 1000, 1500, 0xD157_0003)),
    ("boundary_2d", 2, lambda: boundary_points(2, 600, 800, 0xB0_0002)),
    ("boundary_3d", 3, lambda: boundary_points(3, 600, 800, 0xB0_0003)),
]


def write_points(path: str, P: np.ndarray) -> None:
    with open(path, "wb") as f:
        np.array([len(P)], dtype=np.int32).tofile(f)
        f.write(np.ascontiguousarray(P).tobytes())


def run_distance(dims: int, R: np.ndarray, S: np.ndarray):
    prog = os.path.join(REF_BIN, "dist%d_cpu" % dims)
    with tempfile.TemporaryDirectory() as tmp:
        rp, sp, dp = (os.path.join(tmp, x) for x in ("R.pts", "S.pts", "rows.bin"))
        write_points(rp, R)
        write_points(sp, S)
        out = subprocess.run([prog, rp, sp, dp], cwd=tmp, check=True, stdout=subprocess.PIPE, text=True).stdout
        # init() prints the generator's copy count, join() the match count
        count = int(re.findall(r"^(\d+)$", out, re.M)[-1])
        row = O.POINT_RESULT_DTYPE[3] if dims == 3 else O.REF_CPU_ROW2_DTYPE
        rows = np.fromfile(dp, dtype=row) if os.path.exists(dp) else np.zeros(0, dtype=row)
        return count, rows


def distance_runs() -> list:
    arrays, runs = {}, []
    for case, dims, gen in DIST_CASES:
        R, S = gen()
        count, rows = run_distance(dims, R, S)
        assert len(rows) == count, (case, len(rows), count)
        digest = O.point_rows_digest(rows)
        mine = O.distance_join(dims, R, S)
        assert O.point_rows_digest(mine) == digest, case + ": the oracle differs from the reference"
        arrays[case + "_R"] = np.ascontiguousarray(R).view(np.uint8)
        arrays[case + "_S"] = np.ascontiguousarray(S).view(np.uint8)
        runs.append({"case": case, "dims": dims, "nR": len(R), "nS": len(S), "count": count, "digest": digest})
        print(case, count, digest[:16])
    np.savez_compressed(os.path.join(HERE, "distance.npz"), **arrays)
    return runs


def main() -> None:
    if not os.path.isdir(os.path.join(REF, "joins")):
        sys.exit("make_golden.py: set EJ_REFERENCE to the reference checkout (a directory holding joins/)")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    if "--distance-only" in sys.argv:
        with open(os.path.join(HERE, "reference_runs.json")) as f:
            runs = json.load(f)
        runs["distance"] = distance_runs()
        with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
            json.dump(runs, f, indent=1)
        return
    runs: dict = {"join_ori": {}, "cpu_join": []}

    # 1. join_ori fixture
    j = os.path.join(REF, "joins", "join_ori")
    R = np.fromfile(os.path.join(j, "R"), dtype=np.int32).reshape(-1, 2)
    S = np.fromfile(os.path.join(j, "S"), dtype=np.int32).reshape(-1, 2)
    # keys are the row ids 0..n-1 and vals fit in a byte: store the vals only
    for t in (R, S):
        assert np.array_equal(t[:, 0], np.arange(len(t))) and t[:, 1].min() >= 0 and t[:, 1].max() < 256
    np.savez_compressed(os.path.join(HERE, "join_ori.npz"), R_val=R[:, 1].astype(np.uint8),
                        S_val=S[:, 1].astype(np.uint8))
    with tempfile.TemporaryDirectory() as tmp:
        shutil.copy(os.path.join(j, "R"), tmp)
        shutil.copy(os.path.join(j, "S"), tmp)
        for prog in ("bnlj", "hj", "inner", "outer"):
            out = subprocess.run([os.path.join(REF_BIN, "join_ori_" + prog)], cwd=tmp, check=True,
                                 stdout=subprocess.PIPE, text=True).stdout
            runs["join_ori"][prog] = int(re.findall(r"resultVal: (-?\d+)", out)[0])

    # 2. CPU_JOIN programs on seeded relations
    for prog, name, scale in CASES:
        R, S, _ = relations(name, scale)
        count, rows, diffs, _ = run_cpu_join(prog, R, S)
        entry = {"program": prog, "workload": name, "scale": scale, "nR": len(R), "nS": len(S),
                 "count": count, "checksum": None, "reference_us": diffs}
        if rows is not None:
            assert len(rows) == count, (prog, len(rows), count)
            entry["checksum"] = str(O.checksum(rows))
        runs["cpu_join"].append(entry)
        print(prog, name, scale, count, entry["checksum"], diffs)

    runs["distance"] = distance_runs()
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(runs, f, indent=1)
    print(json.dumps(runs["join_ori"]))


if __name__ == "__main__":
    main()
