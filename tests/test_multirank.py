"""The replicas-only multi-GPU path of bench.py, on CPU: two gloo ranks with
different step times; the job time is the slowest rank's and the throughput
counts both ranks' work."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(REPO))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, world, device="cpu")
    out[rank] = (t, bench.replica_throughput(100.0, t, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = 29500 + os.getpid() % 1000
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        t, v = out[r]
        assert t == 2.0                 # the slower rank
        assert v == 2 * 100.0 / 2.0     # both ranks' units over the max time


def test_single_rank_is_identity():
    sys.path.insert(0, str(REPO))
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_throughput(10.0, 2.0, 1) == 5.0
