"""Multi-GPU runs of the multiply: replicas, one process per GPU.

Row blocks are independent given B, so the path could shard, but nothing here
runs on more than one GPU at a time and no step of the path exchanges data:
`bench.py --gpus N` runs N replicas of the same multiply under torchrun, each
on its own GPU, and reports the whole job as N multiplies in the time of the
slowest rank.  These helpers are that host logic, kept free of CUDA so that
it runs (and is tested) on CPU ranks with the gloo backend.
"""
import os

import torch


def rank_env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest `value` over all ranks (the job's time is its slowest
    rank's); `value` itself when there is no process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, seconds_max, world):
    """Whole-job throughput: every rank processed `units_per_rank` units, the
    job took the slowest rank's `seconds_max`."""
    return world * float(units_per_rank) / float(seconds_max)
