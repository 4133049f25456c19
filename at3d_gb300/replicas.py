"""Several GPUs as independent replicas (one process per GPU, launched by
torchrun).  The solve does not shard: the sweep is a global upwind
dependency per ordinate.  Independent units (wavelengths, requests,
inversion iterates) are spread over the ranks with no collective on the data
path; the only collectives are the barrier and the maximum of the step time
that a measurement takes over the ranks.
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None) -> tuple[int, int]:
    """Join the process group when there is more than one rank (NCCL with a
    GPU, gloo otherwise); returns (rank, world size)."""
    rank, ws, local = world()
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, ws


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(x: float) -> float:
    """The largest value of x over the ranks (x itself with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(n_units: int, rank: int, world_size: int) -> list[int]:
    """The units of one rank: round-robin, so that every unit has exactly
    one rank and ranks differ by at most one unit."""
    return list(range(rank, n_units, world_size))
