"""CPU test of the multi-GPU replica logic of bench.py with two gloo ranks:
each rank builds its own independent batch and seeds, and the whole-job rate
is the units of all ranks over the slowest rank's time."""
import os
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    corr, offsets, sizes, gts, K, seeds = bench.replica_shard("homography", 3, rank)
    seconds = 1.0 + rank  # rank 1 is the slow one
    rate, t = bench.aggregate_rate(3 * 2, seconds, world, dist)
    out[rank] = (float(corr[0, 0]), int(seeds[0]), rate, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_shard_and_aggregate():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29500 + os.getpid() % 1000
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        r0, r1 = out[0], out[1]
    assert r0[0] != r1[0]          # different pairs per rank
    assert (r0[1], r1[1]) == (0, 3)  # disjoint seed ranges
    for r in (r0, r1):
        assert r[3] == pytest.approx(2.0)        # max over ranks
        assert r[2] == pytest.approx(6 * 2 / 2.0)  # all ranks' units / slowest time
