"""The multi-GPU form is independent replicas: bench.py's job time is the slowest rank's and
its value counts every rank's steps.  Checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.replica_time(100.0 * (rank + 1), world, "cpu")  # rank 1 is the slower replica
        out.put((rank, ms, bench.replica_value(ms / 10, world)))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in res:
        assert ms == 200.0                      # the max over ranks, seen by every rank
        assert value == pytest.approx(2 * 1e3 / 20.0)  # both ranks' steps over the slowest time


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_time(12.5, 1, "cpu") == 12.5
    assert bench.replica_value(2.0, 1) == 500.0
