"""Replicas-only multi-GPU path of bench.py, exercised on CPU with gloo:
every rank reports its own timed region, the job reports the slowest, and
each rank builds its own seeded workload."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local = 10.0 + 5.0 * rank
    out[rank] = bench.max_over_ranks(local, world)
    p = bench.blob_problem(6, seed=rank)
    out[world + rank] = float(np.asarray(p["X"]).sum())
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_rank_seeding_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert out[0] == out[1] == 15.0
    assert out[2] != out[3]  # each replica solves its own seeded blob


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
