"""The multi-GPU split of a batch (nsgb.shard): tiles partitioned across ranks by pixel count
with no exchange, and the whole-job figures combined over a world-size-2 gloo group on the CPU
(slowest rank's time, total pixels), as bench.py's batched section does under torchrun."""
import os
import socket

import numpy as np
import pytest


def test_shard_partition_and_balance():
    from nsgb import synth
    from nsgb.shard import rank_tiles, shard_by_cost

    h, w = synth.tile_sizes(256, 256, 4096, 0xC2)
    costs = [int(a) * int(b) for a, b in zip(h, w)]
    for world in (1, 2, 3, 4, 8):
        parts = shard_by_cost(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))  # every tile exactly once
        loads = [sum(costs[i] for i in p) for p in parts]
        # largest-first greedy: no rank exceeds the mean by more than one tile
        assert max(loads) - sum(loads) / world <= max(costs)
        assert all(rank_tiles(costs, world, r) == parts[r] for r in range(world))
    assert shard_by_cost([5, 5, 5], 2) == [[0, 2], [1]]  # ties go to the lower rank and index
    assert shard_by_cost([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        rank_tiles(costs, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from nsgb import synth
        from nsgb.shard import combine, rank_tiles

        h, w = synth.tile_sizes(64, 256, 4096, 7)
        costs = [int(a) * int(b) for a, b in zip(h, w)]
        mine = rank_tiles(costs, world, rank)
        px = sum(costs[i] for i in mine)
        ms, total = combine(10.0 + rank, px)  # rank 1 is the slower one
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        q.put((rank, ms, total, sum(costs), gathered))
    finally:
        dist.destroy_process_group()


def test_combine_over_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, total, all_px, gathered in out:
        assert ms == 11.0  # the slowest rank's time
        assert total == all_px  # the shares add up to the whole batch
        assert sorted(gathered[0] + gathered[1]) == list(range(64)) and not set(gathered[0]) & set(gathered[1])


def test_combine_without_group_is_identity():
    from nsgb.shard import combine

    assert combine(3.5, 42) == (3.5, 42)
