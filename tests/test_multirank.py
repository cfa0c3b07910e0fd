"""The N-rank path of bench.py on CPU (gloo, world size 2): replicas of the
workload, one per rank, no data-path collective; the whole-job value is
all ranks' elements over the slowest rank's step time, and the reference
arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        value, t = bench.whole_job_throughput(1000, 2.0 + rank, world, dist, "cpu")
        ref = bench.reference_arm(None, rank, world) if rank != 0 else "skipped"
        out.put((rank, value, t, ref))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_take_the_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t, ref in res:
        assert t == 3.0                                  # max over ranks (2 ms, 3 ms)
        assert abs(value - world * 1000 / 3.0e-3) < 1e-6
    assert res[1][3] is None                             # rank 1: reference arm returns at once


def test_single_rank_is_the_local_time():
    import bench
    value, t = bench.whole_job_throughput(500, 4.0, 1)
    assert t == 4.0 and value == 500 / 4.0e-3
