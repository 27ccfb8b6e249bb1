"""Independent replicas on several GPUs, one process per GPU.

The reference drives one OpenCL device (FeynSimul/kernel.py:697-700).  Walkers are
independent and the bisection sweep has no exchange step, so N GPUs run N independent
replicas of the walker ensemble with distinct seeds.  The only collectives are host-side:
the final merge of the FP64 accumulators into one ensemble estimate, and the maximum of the
ranks' timings.  They go through torch.distributed (NCCL on GPUs, gloo on CPU) when a process
group is initialised; without one the helpers degrade to the single-process values.
"""
from __future__ import annotations

import numpy as np


def replica_seed(master: int, rank: int) -> int:
    """Master seed of replica ``rank``: distinct for every rank, reproducible."""
    return int((int(master) * 1000003 + 7919 * (int(rank) + 1)) % (2 ** 31 - 1))


class ReplicaGroup:
    """Rank, size and the two collectives of a replica run."""

    def __init__(self):
        self._dist = None
        try:
            import torch.distributed as dist
            if dist.is_available() and dist.is_initialized():
                self._dist = dist
        except ImportError:
            pass
        self.rank = self._dist.get_rank() if self._dist else 0
        self.world = self._dist.get_world_size() if self._dist else 1

    def _tensor(self, values):
        import torch
        dev = "cuda" if self._dist.get_backend() == "nccl" else "cpu"
        return torch.tensor(np.asarray(values, dtype=np.float64), device=dev)

    def max(self, value: float) -> float:
        if not self._dist:
            return float(value)
        t = self._tensor([value])
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def merge(self, per_walker) -> dict:
        """Ensemble mean and standard error over the walkers of all replicas (FP64 sums)."""
        x = np.asarray(per_walker, dtype=np.float64).ravel()
        s = np.array([x.size, x.sum(), np.dot(x, x)])
        if self._dist:
            t = self._tensor(s)
            self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
            s = t.cpu().numpy()
        n, sx, sxx = float(s[0]), float(s[1]), float(s[2])
        mean = sx / n
        var = max(sxx / n - mean * mean, 0.0)
        return {"walkers": int(n), "mean": mean, "se": float(np.sqrt(var / n))}
