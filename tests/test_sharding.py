"""Multi-rank host logic on CPU: partitions, the gloo barrier/max the
benchmark's N > 1 path uses, and the host-staged PSRFITS channel splice
(world size 2, no GPU)."""
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


def channel_products(cc: int, ns: int = 200, nst: int = 4):
    """Fixed per-channel products: the oracle's 8-bit renormalise of seeded
    Stokes for coarse channel cc, and seeded VDIF frame bytes."""
    import numpy as np

    import oracle as O

    rng = np.random.default_rng(1000 + cc)
    S = rng.standard_normal((1, ns, nst, 128)).astype(np.float32) * (1 + cc)
    off, sc, u8 = O.renormalise(S)
    return u8[0], off[0], sc[0], rng.integers(0, 256, (ns, 544), dtype=np.uint8)


def share(channels):
    import numpy as np

    prods = [channel_products(c) for c in channels]
    rows = np.concatenate([p[0] for p in prods], axis=2)        # spliced rows of these channels
    return rows, np.stack([p[1] for p in prods]), np.stack([p[2] for p in prods]), np.stack([p[3] for p in prods])


def _splice_worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import numpy as np

    from sharding import RankContext, gather_splice, shard

    ctx = RankContext(backend="gloo")
    ncc = 5                                   # uneven shares: 3 + 2 channels
    rows, off, sc, vd = share(shard(ncc, ctx.rank, ctx.world))
    out = gather_splice(ctx, ncc, rows, off, sc, vd)
    if ctx.rank == 0:
        full, foff, fsc, fvd = out
        ref = share(range(ncc))               # the one-rank layout
        q.put((0, bool(np.array_equal(full, ref[0]) and np.array_equal(foff, ref[1]) and
                       np.array_equal(fsc, ref[2]) and np.array_equal(fvd, ref[3]))))
    else:
        q.put((ctx.rank, out is None))
    ctx.close()


def test_gloo_splice_equals_one_rank_layout():
    """Two ranks with 3 and 2 of 5 coarse channels: the writer's spliced
    PSRFITS rows, offsets, scales and VDIF frames equal, byte for byte, the
    layout one rank holding all five channels produces."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_splice_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: True, 1: True}


def test_splice_rejects_channels_outside_the_rows():
    import numpy as np

    import vgb

    part = np.zeros((4, 1, 256), np.uint8)
    out = np.zeros((4, 1, 3 * 128), np.uint8)
    with pytest.raises(vgb.VGBError, match="outside"):
        vgb.splice_psrfits(part, 2, 3, out)
