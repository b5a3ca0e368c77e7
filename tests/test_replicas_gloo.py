"""The N>1 path of bench.py without GPUs: N replicas each time their own
copy of the workload, and the job's value is all ranks' particle-steps over
the slowest rank's time, reduced with one scalar collective (here over two
gloo ranks on the CPU)."""
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

    # rank r timed 100*(r+1) ms for (r+1)*1e9 particle-steps
    v, ms = bench.replica_value((rank + 1) * 1e9, 100.0 * (rank + 1), dist, "cpu")
    out.put((rank, v, ms))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_value_over_gloo_ranks(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    total = sum((r + 1) * 1e9 for r in range(world))
    slowest = 100.0 * world
    for _, v, ms in got:
        assert ms == slowest
        assert abs(v - total / (slowest / 1e3)) < 1e-6 * v


def test_single_rank_needs_no_collective():
    import bench

    v, ms = bench.replica_value(2e9, 50.0, None)
    assert ms == 50.0 and v == 2e9 / 0.05
