"""Work partitioning across ranks (one process per GPU).

The path has no data-dependent exchange: coarse channels are independent
(the reference runs one MPI rank per coarse channel, metadata.c:33-48), so
ranks take disjoint contiguous shares of one data-second's coarse channels
(`shard`), each running its own pipeline over its channels, and meet only at
a barrier and a max-of-elapsed-time reduction. The reference's one
collective, the PSRFITS channel splice (MPI_Igather, beam_psrfits.c:608-628),
is the output layout of the renormalise kernel when one GPU holds all
channels, and otherwise `gather_splice`: a host-staged gather of each rank's
finished rows, offsets, scales and VDIF frames to the writer rank over a gloo
group, placed by vgb_splice_psrfits.
"""
from __future__ import annotations

import os

import numpy as np


def shard(n_units: int, rank: int, world: int) -> range:
    """Contiguous block partition of range(n_units); earlier ranks take the
    remainder one unit each."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


class RankContext:
    """RANK / LOCAL_RANK / WORLD_SIZE from the environment (torchrun), a
    process group when WORLD_SIZE > 1 ('nccl' on GPUs, 'gloo' on CPUs), and
    the two operations the benchmark needs."""

    def __init__(self, backend: str | None = None):
        self.rank = int(os.environ.get("RANK", 0))
        self.local_rank = int(os.environ.get("LOCAL_RANK", 0))
        self.world = int(os.environ.get("WORLD_SIZE", 1))
        self.backend = backend
        self._dist = None
        self.host_group = None
        if self.world > 1:
            import torch.distributed as dist

            if backend is None:
                import torch

                backend = "nccl" if torch.cuda.is_available() else "gloo"
            self.backend = backend
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self._dist = dist
            # host buffers travel over gloo whatever the device backend is
            self.host_group = dist.new_group(backend="gloo") if backend != "gloo" else None

    def barrier(self):
        if self._dist is not None:
            self._dist.barrier()

    def max(self, x: float) -> float:
        if self._dist is None:
            return float(x)
        import torch

        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self._dist is None:
            return float(x)
        import torch

        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self._dist is not None and self._dist.is_initialized():
            self._dist.destroy_process_group()


def gather_splice(ctx: RankContext, ncc_total: int, psrfits: np.ndarray, offsets: np.ndarray, scales: np.ndarray,
                  vdif: np.ndarray | None = None, writer: int = 0):
    """The PSRFITS channel splice across ranks, host-staged: each rank holds
    its share shard(ncc_total, rank, world) of the coarse channels as
    spliced rows psrfits [ns][nstokes][ncc_r*128] (uint8), offsets and
    scales [ncc_r][nstokes][128] (float32) and optionally VDIF frames
    [ncc_r][ns][544]; the writer rank receives every share (gloo
    point-to-point, in rank order) and returns the full band's
    [ns][nstokes][ncc_total*128] rows, [ncc_total][nstokes][128] offsets and
    scales and [ncc_total][ns][544] frames; the other ranks return None.
    One rank returns its own buffers."""
    if ctx._dist is None or ctx.world == 1:
        return psrfits, offsets, scales, vdif
    import torch

    import vgb

    dist, group = ctx._dist, ctx.host_group
    send = [psrfits, offsets, scales] + ([vdif] if vdif is not None else [])
    if ctx.rank != writer:
        for a in send:
            dist.send(torch.from_numpy(np.ascontiguousarray(a)), writer, group=group)
        return None
    ns, nst, _ = psrfits.shape
    full = np.empty((ns, nst, ncc_total * vgb.NCHAN), np.uint8)
    off = np.empty((ncc_total, nst, vgb.NCHAN), np.float32)
    scl = np.empty_like(off)
    vd = None if vdif is None else np.empty((ncc_total,) + tuple(vdif.shape[1:]), np.uint8)
    for r in range(ctx.world):
        cr = shard(ncc_total, r, ctx.world)
        if r == writer:
            parts = send
        else:
            n = len(cr)
            parts = [np.empty((ns, nst, n * vgb.NCHAN), np.uint8), np.empty((n, nst, vgb.NCHAN), np.float32),
                     np.empty((n, nst, vgb.NCHAN), np.float32)]
            if vdif is not None:
                parts.append(np.empty((n,) + tuple(vdif.shape[1:]), np.uint8))
            for a in parts:
                dist.recv(torch.from_numpy(a), r, group=group)
        vgb.splice_psrfits(parts[0], cr.start, ncc_total, full)
        off[cr.start:cr.stop] = parts[1]
        scl[cr.start:cr.stop] = parts[2]
        if vd is not None:
            vd[cr.start:cr.stop] = parts[3]
    return full, off, scl, vd
