"""Replicas across processes: one process per GPU, each running its own copy
of the workload.  The explicit step has no data exchange between replicas
(one mesh per GPU; the reference's only collective, the nodal halo sum of a
partitioned mesh, does not arise), so the ranks share nothing but the
bookkeeping of a measurement: a barrier around the timed region, the slowest
rank's time, and sums of per-rank counts.

Rank, world size and local rank come from the torchrun environment (RANK,
WORLD_SIZE, LOCAL_RANK, MASTER_ADDR, MASTER_PORT).  With one process nothing
is initialised; otherwise torch.distributed with NCCL on GPUs or gloo on CPUs.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = None
        self._torch = self._dist = None
        if self.world > 1:
            import torch
            import torch.distributed as tdist

            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            tdist.init_process_group(backend)
            self._torch, self._dist, self.backend = torch, tdist, backend

    @property
    def device(self) -> int:
        """The GPU this rank uses."""
        return self.local if self.world > 1 else 0

    def _tensor(self, x):
        dev = "cuda" if self.backend == "nccl" else "cpu"
        return self._torch.tensor([float(x)], dtype=self._torch.float64, device=dev)

    def barrier(self):
        if self._dist is not None:
            self._dist.barrier()
            if self.backend == "nccl":
                self._torch.cuda.synchronize()

    def max(self, x: float) -> float:
        if self._dist is None:
            return float(x)
        t = self._tensor(x)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self._dist is None:
            return float(x)
        t = self._tensor(x)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self._dist is not None:
            self._dist.destroy_process_group()
            self._dist = None
