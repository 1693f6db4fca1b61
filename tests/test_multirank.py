"""The N>1 host logic of bench.py and the pose sharding, as two gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT
from minibude_gb300.deck import SMALL, shard_deck, shard_range, synthetic_deck


def test_shard_range_covers_exactly_once():
    for n in (0, 1, 7, 65536, 1000003):
        for world in (1, 2, 3, 8):
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, ROOT)
    import oracle
    from bench import Dist
    d = Dist()
    deck = synthetic_deck(SMALL, 0, 96)
    mine = shard_deck(deck, rank, world)
    e = oracle.fasten_f32(mine)
    d.barrier()
    # rank-dependent "step times": the max-reduce must give the slowest rank's
    m = d.max(10.0 + rank)
    import torch
    import torch.distributed as dist
    sizes = [None] * world
    dist.all_gather_object(sizes, e.tolist())
    d.close()
    out.put((rank, m, [x for part in sizes for x in part]))


def test_two_gloo_ranks_barrier_max_and_shard_merge():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import oracle
    full = oracle.fasten_f32(synthetic_deck(SMALL, 0, 96))
    for rank, m, merged in res:
        assert m == 11.0
        assert np.array_equal(np.asarray(merged, np.float32), full)
