"""Replica runs (bench.py --gpus N): the host logic on two CPU ranks (gloo)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from dbd_gb300 import replicas


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = replicas.rank_env()
        assert (r, w, local) == (rank, world, rank)
        dist.barrier()
        t = replicas.max_over_ranks(times[rank], dist)
        out[rank] = (t, replicas.job_rate(1000.0, t, w))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_job_time():
    world = 2
    times = [0.25, 0.5]
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(worker, args=(world, free_port(), times, out), nprocs=world, start_method="spawn")
    for rank in range(world):
        t, rate = out[rank]
        assert t == 0.5
        assert rate == pytest.approx(world * 1000.0 / 0.5)


def test_single_process_needs_no_group():
    assert replicas.max_over_ranks(1.5) == 1.5
    assert replicas.job_rate(10, 2.0, 1) == 5.0
