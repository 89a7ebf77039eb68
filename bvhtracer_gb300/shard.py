"""Work split across GPUs, one process per GPU.

Rays are independent and every BVH is small next to HBM, so the path shards with the BLAS /
TLAS replicated on every GPU and no collective on the data path: a frame splits into contiguous
ray ranges, an uneven batch into whole scenes (greedy longest-processing-time assignment on a
per-scene cost), and results are gathered to rank 0 on the host.  The helpers are plain host
code over torch.distributed (gloo on the host is enough: only the gather crosses processes).
"""
from __future__ import annotations

import numpy as np


def ray_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of rank's share of n rays; shares differ by at most one ray."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    q, r = divmod(int(n), world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def assign_scenes(costs, world: int) -> list[list[int]]:
    """Scene indices per rank: scenes in decreasing cost go to the least-loaded rank (ties to the
    lower rank), each rank's list in increasing index.  Deterministic."""
    costs = np.asarray(costs, np.float64)
    load = np.zeros(world)
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = int(np.argmin(load))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(x) for x in out]


def batch_items_for(items, rays, scene_ids):
    """The sub-batch of `scene_ids`: its items re-based onto a packed copy of their rays."""
    items = np.asarray(items)
    sub = items[list(scene_ids)].copy()
    parts, off = [], 0
    for k in range(len(sub)):
        o, c = int(sub[k]["ray_offset"]), int(sub[k]["ray_count"])
        parts.append(rays[o:o + c])
        sub[k]["ray_offset"] = off
        off += c
    return sub, (np.concatenate(parts) if parts else rays[:0])


def gather_to_rank0(local: np.ndarray, dist, world: int):
    """All ranks' arrays (same dtype) in rank order, concatenated on rank 0 (None elsewhere)."""
    got = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(local, got, dst=0)
    if got is None:
        return None
    return np.concatenate(got) if len(got) else local[:0]


def max_over_ranks(x: float, dist) -> float:
    """The slowest rank's time: the job's time is set by the last GPU to finish."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
