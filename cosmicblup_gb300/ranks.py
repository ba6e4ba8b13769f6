"""Replica ranks: one process per GPU, no data-path collective.

A single MME solve does not shard across GPUs; independent work does (the same
REML workload per GPU, or disjoint subsets of a batch of independent problems).
The ranks only meet on the host, over a gloo process group (torchrun's
RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* environment): a barrier before a timed
region and the maximum of the ranks' times after it, so a whole-job rate is the
units all ranks processed divided by the slowest rank's time.
"""
from __future__ import annotations

import os


def rank_env() -> tuple[int, int, int]:
    """(rank, local_rank, world_size) from the launcher's environment (1 process: 0, 0, 1)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


class Replicas:
    """Host-side coordination of replica ranks over gloo."""

    def __init__(self):
        self.rank, self.local_rank, self.world = rank_env()
        self._dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self._dist = dist

    def barrier(self) -> None:
        if self._dist is not None:
            self._dist.barrier()

    def max(self, x: float) -> float:
        """Maximum of x over the ranks (x itself with one rank)."""
        if self._dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self._dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
        return float(t.item())

    def shard(self, items: list) -> list:
        """This rank's share of independent items (round robin: item i goes to rank i % world)."""
        return list(items[self.rank::self.world])

    def close(self) -> None:
        if self._dist is not None and self._dist.is_initialized():
            self._dist.destroy_process_group()
        self._dist = None


def job_rate(units_per_rank: float, ms_local: float, reps: Replicas) -> tuple[float, float]:
    """(whole-job rate in units per second, slowest rank's ms): every rank processes
    units_per_rank in ms_local milliseconds; the job ends with the slowest rank."""
    ms = reps.max(ms_local)
    total = reps.sum(units_per_rank)
    return total / (ms * 1e-3), ms
