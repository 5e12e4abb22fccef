"""The multi-GPU path is replicas only: every rank runs the same instance and
the bench reports the slowest rank's step and the summed throughput.  The
reduction runs here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        # rank r is slower by r ms; each processes 1000 units per step
        ms, value = bench.replicas_summary(2.0 + rank, 1000.0, dist)
        queue.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(queue.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 3.0
        assert value == pytest.approx(2 * 1000.0 / 3e-3)


def test_single_process_summary():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replicas_summary(4.0, 100.0) == (4.0, 100.0 / 4e-3)
