"""Multi-GPU use of the ray-tracing path: one process per GPU, no collective
on the data path.

Rays are independent and every GPU holds its own copy of the BVH, so work
splits without exchange: a camera pass or ray queue by contiguous ray ranges
(`ray_shard`), a batched multi-mesh launch by whole batches balanced by ray
count (`batch_shard`).  The only collectives are the bench's: a barrier
before the timed region and the maximum of the ranks' step times
(`max_over_ranks`), which is what a whole-job rate divides by.
"""
from __future__ import annotations

import os


def rank_info() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def ray_shard(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of n rays for `rank`; the first n % world ranks
    take one ray more.  The ranges tile [0, n) in rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def batch_shard(ray_counts, world: int) -> list[list[int]]:
    """Assigns whole batches (given their ray counts) to `world` ranks,
    largest first to the least loaded rank (ties to the lower rank), so that
    every rank's launch covers about the same number of rays.  Returns each
    rank's batch indices in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(ray_counts)), key=lambda j: (-int(ray_counts[j]), j)):
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += int(ray_counts[i])
    return [sorted(b) for b in out]


def max_over_ranks(values, device=None) -> list[float]:
    """Element-wise maximum of a list of floats over all ranks (identity
    without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]
