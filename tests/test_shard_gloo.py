"""World-size-2 gloo run of the host sharding logic (CPU): every tree lands
in exactly one shard, the gather restores item order, timing is max over
ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from laml_gb300.shard import shard_bounds


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    from laml_gb300 import shard as S
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items = list(range(n))
    mine = S.shard(items, rank, world)
    scores = [float(-x) for x in mine]          # stand-in per-tree results
    allv = S.gather_scores(scores, n)
    t = S.max_over_ranks(1.0 + rank)
    q.put((rank, mine, allv, t))
    dist.destroy_process_group()


def test_shard_bounds_cover_exactly_once():
    for n in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_bounds(n, r, world)
                seen += list(range(lo, hi))
            assert seen == list(range(n))


def test_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n = 11
    ps = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][1] + out[1][1] == list(range(n))
    for _, _, allv, t in out:
        assert allv == [float(-x) for x in range(n)]
        assert t == 2.0
