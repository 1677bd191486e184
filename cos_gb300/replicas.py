"""Multi-GPU replicas: one process per GPU, each running its own frame.

Every pixel of the Capon path depends only on its own beam's 2K+1 range rows,
so N GPUs need no exchange: each rank processes an independent frame (or a
disjoint slab of beams) and only the timing is combined -- the step time is
the maximum over ranks, the throughput the pixels of all ranks over it.
Launch under torchrun; RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* come from the
environment (use 127.0.0.1 as the master address).
"""
from __future__ import annotations

import os


def env() -> tuple:
    """(rank, local_rank, world_size) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def init(backend: str = "nccl"):
    """Initialise the process group when world_size > 1; returns the
    torch.distributed module or None for a single process."""
    _, _, world = env()
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value: float, device=None) -> float:
    """The maximum of `value` over all ranks (the step time of the slowest)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: int, ms_max: float, world: int) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return units_per_rank * world / (ms_max * 1e-3)


def shard(n: int, rank: int, world: int) -> tuple:
    """Contiguous slab [begin, end) of n beams for `rank` (a frame split across
    GPUs without halo: beams are independent)."""
    return (n * rank) // world, (n * (rank + 1)) // world


def finalize(dist) -> None:
    if dist is not None:
        dist.destroy_process_group()
