"""Replica sharding across GPUs (one process per GPU, no collective on the data path).

The transform is independent per map, so a multi-GPU run splits the maps of a batch
into contiguous shards, one per rank, and each rank runs its own plan on its own GPU.
The only cross-rank steps are host-side: a barrier around timed regions and the
maximum of the ranks' times (or any per-rank scalar).  The reference is single-GPU
(one global instance, SHT.py:16-227); this module has no counterpart there.
"""
from __future__ import annotations


def shard(nmaps: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's maps: contiguous, sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world size {world}")
    if nmaps < 0:
        raise ValueError("nmaps must be >= 0")
    base, extra = divmod(nmaps, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Maximum of a per-rank scalar over the default process group (identity when
    torch.distributed is not initialised).  Works on any backend: the scalar travels
    as a one-element float64 tensor on `device` (CPU for gloo, the rank's GPU for nccl)."""
    if dist is None:
        import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
