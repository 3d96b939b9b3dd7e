"""Replica path of bench.py under torch.distributed: two gloo ranks on the CPU (127.0.0.1), each
with its own timing; both get the maximum, and the job throughput counts every replica's units in
the slowest replica's time."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine = [1.0 + rank, 5.0 - rank]  # rank 0: (1, 5), rank 1: (2, 4)
    ms, kms = bench.max_over_ranks(mine, torch.device("cpu"))
    out[rank] = (ms, kms, bench.job_throughput(1000, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp

    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, kms, tput = res[r]
        assert ms == 2.0 and kms == 5.0
        assert tput == pytest.approx(2 * 1000 / 2e-3)
