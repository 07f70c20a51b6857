"""The multi-rank path of bench.py on CPU: two gloo ranks (replicas) agree on
the slowest rank's time, which is what the whole-job throughput divides by."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.dist_max(1.5 + rank, world, "cpu")
    dist.barrier()
    out.put((rank, t))
    dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2.5), (1, 2.5)]


def test_single_rank_is_identity():
    import bench
    assert bench.dist_max(3.25, 1, "cpu") == 3.25
