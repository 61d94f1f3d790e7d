"""Replicas across GPUs: one process per GPU, each rendering its own share of independent work
(frames of an orbit, jobs of a batch) from its own copy of the inputs.  The path has no exchange
step: ranks meet only to start a timed region together (barrier) and to reduce its timing and
counts (max / sum of scalars).  Launch with torchrun; RANK / WORLD_SIZE / LOCAL_RANK /
MASTER_ADDR / MASTER_PORT come from the environment.

    rep = Replicas()                       # NCCL on GPUs; Replicas(backend="gloo") on CPUs
    for f in rep.shard(64):                # round-robin share of 64 frames
        ...render frame f...
    t = rep.max(local_seconds)
"""
from __future__ import annotations

import os


def shard(n: int, rank: int, world: int) -> list[int]:
    """Round-robin share of items 0..n-1 for `rank`: every item on exactly one rank, shares
    differing by at most one item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, n, world))


def shard_by_cost(costs, rank: int, world: int) -> list[int]:
    """Longest-first greedy share of items with the given costs (e.g. a batch's pixel x step
    estimates): items sorted by decreasing cost go to the least-loaded rank (ties to the lowest
    rank), so that every rank derives the same partition without communication."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += float(costs[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


class Replicas:
    """Process-group plumbing for replica runs (no data-path collective)."""

    def __init__(self, backend: str | None = None, init: bool = True):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend or "nccl"
        self.pg = None
        self._device = "cpu"
        if self.world > 1 and init:
            import torch
            import torch.distributed as dist

            if self.backend == "nccl":
                torch.cuda.set_device(self.local)
                self._device = "cuda"
            dist.init_process_group(self.backend, rank=self.rank, world_size=self.world)
            self.pg = dist

    def shard(self, n: int) -> list[int]:
        return shard(n, self.rank, self.world)

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def _reduce(self, x: float, op) -> float:
        import torch

        t = torch.tensor([x], dtype=torch.float64, device=self._device)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return x if not self.pg else self._reduce(x, self.pg.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return x if not self.pg else self._reduce(x, self.pg.ReduceOp.SUM)

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()
            self.pg = None
