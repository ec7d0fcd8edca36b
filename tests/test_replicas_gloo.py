"""Replica aggregation of bench.py under torch.distributed (two gloo ranks on the CPU).

Every rank solves its own realisation; the job's seconds per solution are the slowest
rank's timed steps divided by the number of solutions (weak scaling).  This covers the
N > 1 host logic without a GPU.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, ms_by_rank, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        out[rank] = bench.job_seconds_per_solution(ms_by_rank[rank], world, device="cpu")
    finally:
        dist.destroy_process_group()


def test_job_seconds_per_solution_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    ms_by_rank = [600.0, 750.0]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, ms_by_rank, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time over the two solutions
    for r in range(2):
        assert out[r] == pytest.approx(0.750 / 2)


def test_job_seconds_per_solution_single():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_seconds_per_solution(612.5, 1) == pytest.approx(0.6125)
