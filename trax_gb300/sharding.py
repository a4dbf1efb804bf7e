"""Multi-GPU data parallelism for the seeding chain: events are independent,
so ranks split a batch into contiguous event ranges balanced by hit count
and run the whole chain on their own range.  No collective touches the data
path; the host only reduces timings and sizes (barrier, max, sum) over
torch.distributed (gloo), one rank per GPU.
"""
from __future__ import annotations

import os
from typing import List, Tuple

import numpy as np


def shard_events(hits_per_event: np.ndarray, world: int) -> List[Tuple[int, int]]:
    """Contiguous [start, end) event ranges, one per rank, balanced by hits.

    Rank r ends where the running hit total first reaches (r+1)/world of the
    whole; every rank gets at least one event while events remain.
    """
    h = np.asarray(hits_per_event, dtype=np.int64)
    n = h.size
    if world <= 0:
        raise ValueError("world must be positive")
    cum = np.cumsum(h)
    total = int(cum[-1]) if n else 0
    cuts = [0]
    for r in range(1, world):
        target = total * r / world
        c = int(np.searchsorted(cum, target, side="left")) + 1
        # this rank gets an event if enough remain; later ranks keep one each
        lo = cuts[-1] + 1 if n - cuts[-1] >= world - r + 1 else cuts[-1]
        hi = max(n - (world - r), lo) if n >= world else n
        cuts.append(min(max(c, lo), hi))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


class Ranks:
    """Rank bookkeeping of one process per GPU (torchrun environment)."""

    def __init__(self, backend: str = "gloo"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if not dist.is_initialized():
                dist.init_process_group(backend, rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def _reduce(self, v: float, op) -> float:
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.MAX) if self.pg else float(v)

    def sum(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.SUM) if self.pg else float(v)

    def close(self):
        if self.pg and self.pg.is_initialized():
            self.pg.destroy_process_group()
