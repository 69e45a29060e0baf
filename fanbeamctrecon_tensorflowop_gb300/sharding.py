"""Batch sharding across ranks (one process per GPU).

Slices are independent, so a global batch splits into contiguous per-rank
ranges with no exchange on the data path; only timing or loss scalars are
reduced.  Works with any torch.distributed backend (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations


def shard_range(batch: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the slices rank ``rank`` of ``world`` owns; the first
    ``batch % world`` ranks take one extra slice."""
    if world <= 0 or not 0 <= rank < world or batch < 0:
        raise ValueError(f"bad shard request batch={batch} rank={rank} world={world}")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a scalar over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
