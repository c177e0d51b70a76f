"""Replica bookkeeping for running the hot path on several GPUs of one node.

The resident light-stack path has no exchange step: every GPU integrates its
own stack (frames and output pixels are independent), so several GPUs are
independent replicas.  torch.distributed only provides the barrier around the
timed region and the max-over-ranks time; no data moves between ranks.
"""

from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init(backend: str, device=None) -> None:
    """Joins the process group when WORLD_SIZE > 1 (env:// rendezvous)."""
    import torch.distributed as dist

    if dist.is_available() and not dist.is_initialized() and dist_env()[1] > 1:
        if device is not None and backend == "nccl":
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the slowest replica sets the time)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, units_per_rank_per_step: float, steps: int, slowest_seconds: float) -> float:
    """Whole-job throughput: the units every rank processed / the slowest rank's time."""
    if slowest_seconds <= 0.0:
        raise ValueError("elapsed time must be positive")
    return world * units_per_rank_per_step * steps / slowest_seconds


def shutdown() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
