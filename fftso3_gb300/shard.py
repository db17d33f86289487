"""Function-batch sharding across GPUs (one process per GPU).

The transforms of different functions are independent, so a batch shards by
function with no exchange step: each rank transforms its own contiguous block
of functions on its own GPU, and only host-side bookkeeping (timing, optional
result collection) crosses ranks.  These helpers hold that bookkeeping; they
use torch.distributed when a process group is initialised (NCCL on GPUs, gloo
for tests on the CPU) and are no-ops otherwise.
"""
from __future__ import annotations

import numpy as np


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def rank_world() -> tuple[int, int]:
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def partition(n_functions: int, world: int, rank: int) -> range:
    """Contiguous block of the functions owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world or n_functions < 0:
        raise ValueError("bad partition arguments")
    base, extra = divmod(n_functions, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float) -> float:
    """The maximum of a per-rank scalar (e.g. a step time) over all ranks."""
    d = _dist()
    if d is None:
        return float(value)
    import torch

    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(local: np.ndarray, n_functions: int):
    """Concatenate every rank's block (shape (len(partition), ...)) on rank 0 in function order;
    other ranks get None."""
    d = _dist()
    if d is None:
        return local
    import torch

    rank, world = d.get_rank(), d.get_world_size()
    parts = [None] * world
    d.all_gather_object(parts, (rank, np.asarray(local)))
    if rank != 0:
        return None
    parts.sort(key=lambda x: x[0])
    out = np.concatenate([p for _, p in parts], axis=0)
    if out.shape[0] != n_functions:
        raise RuntimeError("gathered blocks do not cover the batch")
    return out
