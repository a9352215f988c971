"""Work partitioning across ranks (one process per GPU).

The path has no data-dependent exchange: coarse channels and seconds are
independent (the reference runs one MPI rank per coarse channel,
metadata.c:33-48), so ranks take disjoint shares of the units and meet only
at a barrier and a max-of-elapsed-time reduction. The reference's one
collective, the PSRFITS channel splice (MPI_Igather, beam_psrfits.c:608-628),
is the output layout of the renormalise kernel when one GPU holds all
channels, and a host-side gather of finished rows otherwise.
"""
from __future__ import annotations

import os


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
        if self.world > 1:
            import torch.distributed as dist

            if backend is None:
                import torch

                backend = "nccl" if torch.cuda.is_available() else "gloo"
            self.backend = backend
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self._dist = dist

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
