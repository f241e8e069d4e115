"""Build the engine's shared library in-tree with nvcc for sm_103a.

Each CUDA translation unit under ``csrc/`` is compiled in parallel into
``_build/`` and linked into ``eating_one_gb300/libeating_one.so``.  The build is
incremental: nothing is recompiled when the library is newer than every
source and header.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libeating_one.so")
CLI_PATH = os.path.join(PKG_DIR, "ej_join")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", INCLUDE, "-I", CSRC,
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the join engine")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    files = []
    for d in (CSRC, INCLUDE):
        files += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    return files


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (proc.returncode, " ".join(cmd), proc.stdout))


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every CUDA source and link the shared library; returns its path."""
    deps = _deps()
    if not force and not _stale(LIB_PATH, deps) and not _stale(CLI_PATH, deps):
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    for src in _sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        _run(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
        objs = list(pool.map(compile_one, jobs))
    tmp = LIB_PATH + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB_PATH)
    # the reference-style command-line driver, linked against the library
    cli_src = os.path.join(PKG_DIR, "cli", "ej_join.cpp")
    if os.path.exists(cli_src):
        _run([nvcc, "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI_PATH + ".tmp",
              "-L", PKG_DIR, "-leating_one", "-Xlinker", "-rpath,$ORIGIN"])
        os.replace(CLI_PATH + ".tmp", CLI_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
