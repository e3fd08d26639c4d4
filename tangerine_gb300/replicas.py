"""Replica runs across ranks: one process per GPU, each exporting its own copy of the work.

The path has no data exchange between GPUs (models, bricks and lattice points are
independent), so ranks share only what the measurement needs: a barrier around the timed
region, the slowest rank's time, and summed unit counts.  `shard` splits a list of
independent items (models of a batch) across ranks when a run wants the work divided
instead of replicated.  NCCL carries these on GPUs; gloo on the CPU (the tests run two
ranks that way).
"""

from __future__ import annotations

import os


def shard(items, rank: int, world: int):
    """Items rank, rank + world, rank + 2*world, ...: disjoint, together all of them."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside a world of {world}")
    return items[rank::world]


class Replicas:
    """Process group of a replica run (none when world == 1)."""

    def __init__(self, world: int | None = None, rank: int | None = None, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1")) if world is None else int(world)
        self.rank = int(os.environ.get("RANK", "0")) if rank is None else int(rank)
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if not dist.is_initialized():
                dist.init_process_group(backend, world_size=self.world, rank=self.rank)
            self.dist = dist
            self.device = "cuda" if backend == "nccl" else "cpu"

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, value: float, op) -> float:
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, value: float) -> float:
        """The largest value over ranks (the slowest rank's time)."""
        return float(value) if self.dist is None else self._reduce(value, self.dist.ReduceOp.MAX)

    def sum(self, value: float) -> float:
        """The sum over ranks (units processed by the whole job)."""
        return float(value) if self.dist is None else self._reduce(value, self.dist.ReduceOp.SUM)

    def close(self) -> None:
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()
        self.dist = None
