"""Host logic for running the path on several GPUs of one node.

Profiles are independent (the reference runs them in parallel with no
reduction, src/CRTM_Forward_Module.f90:402-414), so a batch is split into
contiguous profile ranges, one per rank, with no collective on the data path.
The only collectives are the timing reductions of the benchmark.
"""
from __future__ import annotations

from typing import Tuple


def shard_profiles(n_profiles: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of the profiles rank ``rank`` of ``world`` handles: contiguous
    ranges whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    base, extra = divmod(n_profiles, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The maximum of ``value`` over all ranks (identity without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
