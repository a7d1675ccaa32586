"""Replica bookkeeping for runs on several GPUs of one node.

Scans are independent, so N GPUs run N replicas: rank r reconstructs its own
scan (seeded with seed + 1000 r) with no collective on the data path.  The
only collectives are the ones a job-level measurement needs: a barrier
around the timed region, the maximum time over ranks and the sum of the work
(pairs) over ranks.  NCCL on GPUs; gloo (CPU tensors) for the host-side tests.
"""
from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(seed: int, rank: int) -> int:
    return seed + 1000 * rank


class Replicas:
    def __init__(self, backend: str | None = None):
        self.rank, self.world, self.local = env()
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch.distributed as dist

            backend = backend or "nccl"
            dist.init_process_group(backend)
            self.dist = dist
            self.device = "cuda" if backend == "nccl" else "cpu"

    def _reduce(self, x: float, op) -> float:
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def barrier(self) -> None:
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        return self._reduce(x, self.dist.ReduceOp.MAX) if self.dist else float(x)

    def sum(self, x: float) -> float:
        return self._reduce(x, self.dist.ReduceOp.SUM) if self.dist else float(x)

    def job_rate(self, units: float, ms: float) -> float:
        """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
        return self.sum(units) / (self.max(ms) / 1000.0)

    def close(self) -> None:
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None
