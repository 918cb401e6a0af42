"""Placement of batch and serving work on several GPUs.

Every image is an independent max-flow, so a job shards by image: each rank
solves its own images on its own GPU and nothing crosses ranks on the data
path.  The only collectives are host-side bookkeeping: the max of the ranks'
step times (the job's time), sums of pixel counts, and gathering small
per-image results (flows) for checking.  A single image is never split
across GPUs.

Two placements:
  * weak scaling (the benchmark): every rank solves its own batch of the
    same distribution, the images of rank r seeded after those of rank r-1;
  * strong scaling (one fixed batch over N ranks): longest-processing-time
    partition of the images by pixel count, so the ranks' loads differ by at
    most one image.
Collectives go through torch.distributed (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import heapq


def lpt_partition(sizes, world: int):
    """Indices of `sizes` split into `world` lists, largest first onto the
    least loaded rank (ties: the lowest rank).  Deterministic."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(p) for p in parts]


def rank_share(sizes, rank: int, world: int):
    """This rank's image indices under the strong-scaling placement."""
    return lpt_partition(sizes, world)[rank]


def weak_seed0(seed0: int, n_images: int, rank: int) -> int:
    """First image seed of `rank` when every rank solves its own batch of
    n_images: ranks get disjoint, consecutive seed ranges."""
    return seed0 + rank * n_images


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def _reduce(v: float, op_name: str, device=None) -> float:
    dist = _dist()
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(v: float, device=None) -> float:
    """The job's time of a step: the slowest rank's."""
    return _reduce(v, "MAX", device)


def sum_over_ranks(v: float, device=None) -> float:
    return _reduce(v, "SUM", device)


def gather(obj):
    """Every rank's `obj`, in rank order (a list of one without a process group)."""
    dist = _dist()
    if dist is None:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def barrier():
    dist = _dist()
    if dist is not None:
        dist.barrier()
