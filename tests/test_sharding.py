"""Multi-rank host logic on CPU: partitions and the gloo barrier/max the
benchmark's N > 1 path uses (world size 2, no GPU)."""
import os
import socket

import pytest

from sharding import shard


def test_shard_covers_disjointly():
    for n in (0, 1, 7, 24, 25):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            flat = [u for p in parts for u in p]
            assert flat == list(range(n))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from sharding import RankContext, shard

    ctx = RankContext(backend="gloo")
    mine = shard(24, ctx.rank, ctx.world)
    ctx.barrier()
    elapsed = 1.5 + ctx.rank          # a per-rank "time"
    q.put((ctx.rank, list(mine), ctx.max(elapsed), ctx.sum(len(mine))))
    ctx.close()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, m0, t0), (r1, s1, m1, t1) = out
    assert s0 + s1 == list(range(24)) and not set(s0) & set(s1)
    assert m0 == m1 == 2.5           # max over ranks
    assert t0 == t1 == 24            # every unit processed once
