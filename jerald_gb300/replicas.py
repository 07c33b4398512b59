"""Replica runs of the fused LDL step on several GPUs of one box.

At world size > 1 the reference decomposes the mesh into slabs and moves
particles to their owners with an Alltoallv (lib/parops_fast.h:52-351) and
transposes slabs inside FFTW-MPI (lib/parfft.h:33-76).  One GPU holds a whole
512^3 (22 GB) or 1024^3 (~155 GB with recomputed force meshes) box, so the
GPU build runs independent replicas instead: rank r evaluates its own box
(seed r) with no data-path collective.  Only the timing is combined, as the
maximum over ranks, so the aggregate throughput counts every rank's steps
over the slowest rank's clock.
"""
from __future__ import annotations

import os

import torch


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _dist_ready() -> bool:
    import torch.distributed as dist
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def max_over_ranks(x: float, device=None) -> float:
    """Maximum of a per-rank scalar over the process group (the value itself
    without one).  `device` is where the reduction buffer lives: a CUDA
    device for NCCL, None (CPU) for gloo."""
    if not _dist_ready():
        return float(x)
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(ms_per_step: float, device=None) -> tuple[float, float]:
    """(steps/s summed over all replicas, the slowest replica's ms/step)."""
    ms = max_over_ranks(ms_per_step, device)
    n = 1
    if _dist_ready():
        import torch.distributed as dist
        n = dist.get_world_size()
    return n * 1000.0 / ms, ms


def replica_seed(rank: int, base: int = 0) -> int:
    """Seed of rank r's synthetic box: replicas evaluate different boxes."""
    return base + rank
