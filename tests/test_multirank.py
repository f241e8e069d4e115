"""The multi-GPU bench path on CPU: world_size-2 gloo ranks.

The engine runs one process per GPU with independent replicas (weak scaling,
no data-path collective); bench.py only gathers every rank's step time and
reports the whole job at the slowest rank's pace.  This runs that gather and
aggregation over two gloo ranks on 127.0.0.1."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    per_rank = bench.gather_ms(ms, dist, torch.device("cpu"))
    value, ms_max = bench.aggregate(per_rank, units_per_rank=1000.0, steps=1)
    q.put((rank, per_rank, value, ms_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_at_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, per_rank, value, ms_max in results:
        assert per_rank == [10.0, 15.0]
        assert ms_max == 15.0
        assert value == pytest.approx(2 * 1000.0 / 0.015)


def test_single_process_aggregate():
    import bench

    assert bench.gather_ms(3.0, None, None) == [3.0]
    assert bench.aggregate([4.0], 100.0, 1) == (100.0 / 0.004, 4.0)
