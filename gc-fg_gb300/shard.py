"""Placement of batch and serving work on several GPUs.

Every image is an independent max-flow, so a job shards by image: each rank
solves its own images on its own GPU and nothing crosses ranks on the data
path.  The only collectives are host-side bookkeeping: the max of the ranks'
step times (the job's time), sums of pixel counts, and gathering small
per-image results (flows) for checking.  A single image is never split
across GPUs.

Three placements:
  * weak scaling (the benchmark): every rank solves its own batch of the
    same distribution, the images of rank r seeded after those of rank r-1;
  * strong scaling (one fixed batch over N ranks): longest-processing-time
    partition of the images by pixel count, so the ranks' loads differ by at
    most one image;
  * serving (RequestRouter): one server per GPU; a new image goes to the GPU
    with the least device state, a scribble edit to the GPU that holds its
    image.
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


# Device bytes a resident image holds per 32x32 tile in a server: the tile
# arena (capacities 16 KB, excess and heights 8 KB, border heights 512 B,
# neighbour table, finite-height and reach rows, six mask planes, counters,
# marks, owner) plus its pixels' RGB, scribble and two label maps (6 B each).
# The server admits images by the same figure (csrc/serve.cu, TILE_BYTES).
SERVE_TILE_BYTES = 16384 + 2 * 4096 + 512 + 16 + 128 + 128 + 768 + 4 + 8 + 12 + 1024 * 6


def image_footprint(width: int, height: int) -> int:
    """Device bytes of one resident image in a server."""
    return ((int(width) + 31) // 32) * ((int(height) + 31) // 32) * SERVE_TILE_BYTES


class RequestRouter:
    """Host-side dispatcher of segmentation requests over several GPUs, one
    server (gcfg_serve_*) per GPU; no data crosses GPUs.

    * A new image goes to the GPU whose server holds the least device state
      (resident images plus requests in flight, in bytes), among the GPUs
      whose memory cap still holds it; when none does, to the least loaded
      one (its server then evicts idle images, least recently used first).
      Ties go to the lowest rank, so placement is deterministic.
    * A scribble edit goes to the GPU that holds its image: the residual
      graph and flow the warm re-solve starts from are resident there.
    * done() and release() keep the loads current when a request completes
      and when a server drops an image (released or evicted)."""

    def __init__(self, world: int, mem_cap_bytes: int):
        if world < 1:
            raise ValueError("world must be >= 1")
        self.world = world
        self.cap = int(mem_cap_bytes)
        self.resident = [0] * world
        self.inflight = [0] * world
        self.owner = {}
        self.size = {}

    def load(self, rank: int) -> int:
        return self.resident[rank] + self.inflight[rank]

    def place_new(self, session, width: int, height: int) -> int:
        """Rank that serves new image `session`; its request counts as in flight."""
        if session in self.owner:
            raise ValueError(f"session {session} already placed")
        fp = image_footprint(width, height)
        if fp > self.cap:
            raise ValueError(f"image {width}x{height} needs {fp} bytes, more than one server's cap {self.cap}")
        fits = [r for r in range(self.world) if self.resident[r] + fp <= self.cap]
        r = min(fits or range(self.world), key=lambda k: (self.load(k), k))
        self.owner[session] = r
        self.size[session] = fp
        self.resident[r] += fp
        self.inflight[r] += fp
        return r

    def place_edit(self, session) -> int:
        """Rank that holds `session` (KeyError when it was never placed or was released)."""
        r = self.owner[session]
        self.inflight[r] += self.size[session]
        return r

    def done(self, session):
        """A request of `session` completed."""
        r = self.owner[session]
        self.inflight[r] -= self.size[session]

    def release(self, session):
        """The server dropped `session` (released or evicted)."""
        r = self.owner.pop(session)
        self.resident[r] -= self.size.pop(session)
