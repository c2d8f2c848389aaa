"""Replicas across GPUs: one process per GPU, tracks are independent, so a
batch is split by rank with no data-path collective.  The only collectives are
timing ones (max of the per-rank elapsed time, sum of the units processed),
which run on whatever process group the caller initialised (NCCL on GPUs,
gloo on CPU).

The reference tracks one person per process (the ROS node of src/pfPoseTracker.cpp); a
multi-person or multi-camera deployment runs independent trackers, which is
exactly what a rank here is.
"""
from __future__ import annotations

import heapq
import os


def dist_env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seed(base_seed: int, rank: int) -> int:
    """Seed of rank r's synthetic batch under weak scaling (fixed work per GPU)."""
    return int(base_seed) + 1000 * int(rank)


def shard_by_work(costs, world_size: int):
    """Split track indices over ranks, balancing the summed cost (e.g. particles
    x frames) by longest-processing-time-first; deterministic (ties by index).
    Returns a list of sorted index lists, one per rank."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world_size)]
    heapq.heapify(heap)
    out = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in out]


def _collective(value: float, op_name: str, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = device if device is not None else ("cuda" if dist.get_backend() == "nccl" else "cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(seconds: float, device=None) -> float:
    """The job's time: the slowest rank's."""
    return _collective(seconds, "MAX", device)


def sum_over_ranks(units: float, device=None) -> float:
    return _collective(units, "SUM", device)


def whole_job_rate(units_this_rank: float, seconds_this_rank: float, device=None) -> float:
    """Units processed by all ranks / max over ranks of the elapsed time."""
    return sum_over_ranks(units_this_rank, device) / max_over_ranks(seconds_this_rank, device)
