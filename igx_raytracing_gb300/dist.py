"""Multi-GPU helpers: the ray-query path shards by ray index.

Every ray is independent (its result depends only on its scene and itself),
so N GPUs each hold a replica of the scene and trace a contiguous range of
the rays (trace_sharded); results land in disjoint slices and no collective
touches the traversal.  A caller that wants the whole batch's results on
every rank gathers the slices once at the end (trace_sharded's `gather`).
The benchmark runs replicas instead (every rank traces the whole step: weak
scaling), and its only collective is the timing reduction (the slowest rank
defines the step time).
"""
from __future__ import annotations

import numpy as np


def trace_sharded(trace, rays, prev_hit=None, gather: bool = True, rank: int | None = None,
                  world: int | None = None):
    """Traces this rank's contiguous slice of `rays` (and of `prev_hit`) with
    `trace(rays, prev_hit)` -- e.g. Scene.trace_geometry or
    Scene.trace_occlusion of this rank's replica of the scene -- and returns
    (results, begin, end).  With `gather`, results is the whole batch's,
    assembled on every rank from the ranks' slices in rank order (one
    all_gather of host arrays over the default process group); otherwise it
    is this rank's slice [begin, end).  rank / world default to the process
    group's (1 rank without one)."""
    import torch.distributed as dist

    grouped = dist.is_available() and dist.is_initialized()
    if rank is None:
        rank = dist.get_rank() if grouped else 0
    if world is None:
        world = dist.get_world_size() if grouped else 1
    begin, end = shard_range(len(rays), rank, world)
    part = trace(rays[begin:end], None if prev_hit is None else prev_hit[begin:end])
    if not gather or world == 1:
        return part, begin, end
    parts = [None] * world
    dist.all_gather_object(parts, np.ascontiguousarray(part))
    return np.concatenate(parts), 0, len(rays)


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of n items for `rank` of `world`; the first
    n % world ranks take one extra item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
