"""Multi-GPU bookkeeping for replicated propagation (one process per GPU).

The propagation path has no data-path exchange between independent
instances, so several GPUs run disjoint work and only timing is combined:
every rank propagates its own instances (a single model is replicated; a batched
sweep gives each rank its own seeded shard, so per-GPU work is fixed: weak
scaling), and the job's throughput is the units of all ranks divided by the
slowest rank's time.  No collective touches the state.
"""
from __future__ import annotations

import os


def env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_seed(base_seed: int, rank: int) -> int:
    """Seed of rank `rank`'s shard of a seeded batched sweep (rank 0 keeps the base seed)."""
    return base_seed + 1000003 * rank


def job_throughput(units_this_rank: float, seconds_this_rank: float, group=None):
    """(units per second over all ranks, slowest rank's seconds).

    Sums the units and takes the maximum time over the process group (two
    scalar all-reduces on the host's group), so the figure is whole-job
    throughput measured against the slowest replica."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return units_this_rank / seconds_this_rank, seconds_this_rank
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else "cpu"
    u = torch.tensor([float(units_this_rank)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds_this_rank)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()) / float(t.item()), float(t.item())
