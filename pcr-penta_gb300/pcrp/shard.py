"""Batch sharding across GPUs: one process per GPU, contiguous ranges of
systems, no collective on the data path.

Systems are independent (the reference's grid is over systems, main.cu:49),
so a multi-GPU solve is a set of replicas, each solving its own contiguous
range of systems; the only optional communication is gathering results.
"""
from __future__ import annotations

from typing import Tuple


def shard_range(m: int, world: int, rank: int) -> Tuple[int, int]:
    """[j0, j1) of the m systems owned by `rank` of `world` (balanced, contiguous)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    if m < 0:
        raise ValueError("negative batch")
    base, extra = divmod(m, world)
    j0 = rank * base + min(rank, extra)
    return j0, j0 + base + (1 if rank < extra else 0)


def local_view(arrs, m: int, n: int, world: int, rank: int):
    """Slices of the six contiguous-layout arrays belonging to `rank`."""
    j0, j1 = shard_range(m, world, rank)
    return [v[j0 * n: j1 * n] for v in arrs], j1 - j0


def solve_f64_sharded(arrs, m: int, n: int, world: int, rank: int, stream=None, opts=None) -> int:
    """Solve this rank's share of a contiguous batch in place; returns its system count."""
    from . import solve_f64
    local, ml = local_view(arrs, m, n, world, rank)
    if ml:
        solve_f64(*local, ml, n, opts=opts, stream=stream)
    return ml
