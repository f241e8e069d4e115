"""eating_one_gb300 - a GB300-native relational join engine (sm_103a).

The join entry points of yabuta/eating_one (radix hash join, build-side-only
hash join, block nested-loop join, hash-index and sort-index joins, left outer
join, 3-way star join) over TUPLE{int key, int val} relations, as hand-written
CUDA kernels behind the C ABI of include/ej.h (libeating_one.so).  This
package holds the build script, the ctypes binding and a thin torch-tensor
mirror of the ABI (engine.Engine).
"""
from .build import build  # noqa: F401

__all__ = ["build", "Engine", "JoinError", "workload"]


def __getattr__(name):
    if name in ("Engine", "JoinError", "Index"):
        from . import engine
        return getattr(engine, name)
    if name == "workload":
        from .workloads import workload
        return workload
    raise AttributeError(name)
