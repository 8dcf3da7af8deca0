"""Multi-GPU path of bench.py on CPU: replicas only (no data-path collective).

Each rank advances its own replica; the only exchange is the max over ranks of the
timings, done here by two gloo processes.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank 1 is the slower replica: both ranks see its times
    mine = [100.0 + 50.0 * rank, 120.0 - 10.0 * rank]
    got = bench.reduce_max(mine, dist)
    value = bench.job_value(1000, 10, world, got[0])
    q.put((rank, got, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in res:
        assert got == [150.0, 120.0]
        # 2 replicas x 1000 particles x 10 steps in the slowest rank's 150 ms
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)


def test_job_value_scales_with_replicas():
    import bench

    assert bench.job_value(340050, 10, 4, 250.0) == pytest.approx(4 * bench.job_value(340050, 10, 1, 250.0))
