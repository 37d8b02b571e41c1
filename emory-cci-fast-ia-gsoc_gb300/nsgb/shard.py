"""Partition of a batch of independent tiles across ranks (one process per GPU).

The tiles of a batch share nothing (each is its own reconstruction and labelling), so a
multi-GPU run needs no data exchange: every rank prepares and runs its own nsgb_chain_batch
on its share, and only the timing and pixel totals are combined.  Tiles go to ranks by pixel
count, largest first, each onto the rank with the fewest pixels so far (ties to the lower rank);
the result depends only on the costs and the number of ranks, so every rank computes the same
partition without communicating.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def shard_by_cost(costs: Sequence[int], world: int) -> List[List[int]]:
    """Tile indices per rank (each list in ascending order)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    loads = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-int(costs[k]), k)):
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(i)
        loads[r] += int(costs[i])
    return [sorted(p) for p in parts]


def rank_tiles(costs: Sequence[int], world: int, rank: int) -> List[int]:
    """The tile indices this rank runs."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return shard_by_cost(costs, world)[rank]


def combine(ms: float, px: int, group=None) -> Tuple[float, int]:
    """Whole-job figures over the ranks of the default process group: the slowest rank's time
    and the total pixels (the job ends when the last rank does).  Without a process group (one
    rank) the inputs come back unchanged."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return ms, px
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    n = torch.tensor([px], dtype=torch.int64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), int(n.item())
