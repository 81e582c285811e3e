"""bench.py with N > 1 runs one replica per rank (the 3D dam break is one
domain; nothing is exchanged) and reports the job's time as the maximum over
the ranks: the cross-rank reduction checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, dist, "cpu")
    finally:
        dist.destroy_process_group()


def test_time_is_the_slowest_rank():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_keeps_its_value():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
