"""The multi-rank (replica) aggregation of bench.py on CPU with gloo,
world size 2: the job's step time is the slowest rank's, its throughput
all ranks' cells over that time."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    t = bench.slowest_rank_time(1.5 + rank, dist, "cpu")  # rank 1 is the slow one
    out[rank] = (r, w, local, t, bench.job_mlups(1000000, w, t))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_sets_the_job_time_world_2():
    world = 2
    port = _free_port()
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for rank in range(world):
        r, w, local, t, mlups = out[rank]
        assert (r, w, local) == (rank, world, rank)
        assert t == 2.5
        assert mlups == pytest.approx(2 * 1000000 / 2.5e-3 / 1e6)


def test_single_process_keeps_its_time():
    assert bench.slowest_rank_time(3.25, None, "cpu") == 3.25
    assert bench.job_mlups(134217728, 1, 2.95) == pytest.approx(134217728 / 2.95e-3 / 1e6)
