"""Independent replicas on several GPUs, one process per GPU.

The reference drives one OpenCL device (FeynSimul/kernel.py:697-700).  Walkers are
independent and the bisection sweep has no exchange step, so N GPUs run N independent
replicas of the walker ensemble with distinct seeds.  The only collectives are host-side:
the final merge of the accumulators into one ensemble estimate (operator means, correlator
means, histogram and bin counts, accepts), and the maximum of the ranks' timings.  They go
through torch.distributed (NCCL on GPUs, gloo on CPU) when a process group is initialised;
without one the helpers degrade to the single-process values.

Means and variances are merged from per-rank (count, mean, M2) triples with the pairwise
update of Chan, Golub and LeVeque ("Updating formulae and a pairwise algorithm for
computing sample variances", 1979): no sum of squares of the raw values is formed, so an
observable with a large mean and a small spread keeps its variance.  The ranks' triples
are combined in rank order on every rank, so every rank holds the same result bit for bit.
"""
from __future__ import annotations

import numpy as np


def replica_seed(master: int, rank: int) -> int:
    """Master seed of replica ``rank``: distinct for every rank, reproducible."""
    return int((int(master) * 1000003 + 7919 * (int(rank) + 1)) % (2 ** 31 - 1))


def moments(x) -> tuple:
    """(n, mean, M2) per column of x [samples, k] (or of a 1-D x), FP64, M2 = sum of squared
    deviations from the mean (two passes)."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    n = float(x.shape[0])
    mean = x.mean(axis=0) if n else np.zeros(x.shape[1])
    d = x - mean
    return n, mean, np.einsum("ij,ij->j", d, d)


def chan_combine(parts) -> tuple:
    """Combine [(n, mean, M2), ...] (each mean / M2 an array over the same columns) in order:
    delta = mean_b - mean_a, mean = mean_a + delta n_b / n, M2 = M2_a + M2_b + delta^2 n_a n_b / n."""
    n, mean, m2 = parts[0]
    mean, m2 = np.array(mean, dtype=np.float64), np.array(m2, dtype=np.float64)
    for nb, mb, m2b in parts[1:]:
        if nb == 0:
            continue
        tot = n + nb
        delta = np.asarray(mb) - mean
        mean = mean + delta * (nb / tot)
        m2 = m2 + np.asarray(m2b) + delta * delta * (n * nb / tot)
        n = tot
    return n, mean, m2


class ReplicaGroup:
    """Rank, size and the collectives of a replica run."""

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

    def _device(self):
        return "cuda" if self._dist.get_backend() == "nccl" else "cpu"

    def _tensor(self, values, dtype=np.float64):
        import torch
        return torch.tensor(np.asarray(values, dtype=dtype), device=self._device())

    def max(self, value: float) -> float:
        if not self._dist:
            return float(value)
        t = self._tensor([value])
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, value: float) -> float:
        """Sum of a float over the ranks (FP64)."""
        if not self._dist:
            return float(value)
        t = self._tensor([value])
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
        return float(t.item())

    def sum_counts(self, counts) -> np.ndarray:
        """Element-wise sum over the ranks of integer counts (histogram and bin counts,
        accepts), exact in int64."""
        c = np.asarray(counts).astype(np.int64)
        if not self._dist:
            return c
        t = self._tensor(c, np.int64)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM)
        return t.cpu().numpy().astype(np.int64)

    def gather_moments(self, x) -> tuple:
        """(n, mean, M2) per column over the samples of all ranks (Chan's update, rank order)."""
        n, mean, m2 = moments(x)
        if not self._dist:
            return n, mean, m2
        import torch
        k = mean.shape[0]
        mine = self._tensor(np.concatenate([[n], mean, m2]))
        bufs = [torch.empty_like(mine) for _ in range(self.world)]
        self._dist.all_gather(bufs, mine)
        parts = []
        for b in bufs:
            v = b.cpu().numpy()
            parts.append((float(v[0]), v[1:1 + k], v[1 + k:]))
        return chan_combine(parts)

    def merge(self, per_walker) -> dict:
        """Ensemble mean and standard error of one per-walker observable over the walkers of
        all replicas."""
        n, mean, m2 = self.gather_moments(np.asarray(per_walker, dtype=np.float64).ravel())
        var = m2[0] / n if n else 0.0
        return {"walkers": int(n), "mean": float(mean[0]), "se": float(np.sqrt(var / n)) if n else 0.0}

    def merge_kernel(self, k) -> dict:
        """Every accumulator of a PIMCKernel merged over the replicas: per operator the
        ensemble mean and standard error of the per-walker means (kernel.py:576-606), the
        correlator's per-lag mean and standard error over the walkers (kernel.py:608-617),
        the summed histogram and bin counts (kernel.py:619-637), and the acceptance rate
        from the summed accepts (kernel.py:648-658).  Parts the kernel was not built with
        are left out."""
        out = {"replicas": self.world}
        if getattr(k, "_enableOperator", False):
            ops = np.asarray(k.getOperators(), dtype=np.float64)          # (nOps, walkers)
            n, mean, m2 = self.gather_moments(ops.T)
            out["operators"] = {"walkers": int(n), "mean": mean.tolist(),
                                "se": np.sqrt(m2 / n / n).tolist()}
        if getattr(k, "_enableCorrelator", False):
            vals = k.getCorrelatorPerWalker()                               # (walkers, nCorr, N/2)
            shape = vals.shape[1:]
            n, mean, m2 = self.gather_moments(vals.reshape(vals.shape[0], -1))
            out["correlator"] = {"walkers": int(n), "mean": mean.reshape(shape),
                                 "se": np.sqrt(m2 / n / n).reshape(shape)}
        if getattr(k, "_histBins", 0):
            _, counts = k.getHistogram(density=False)
            out["histogram_counts"] = self.sum_counts(counts)
        if getattr(k, "_enableBins", False):
            out["bin_counts"] = self.sum_counts(k.getBinCountsRaw())
        acc = np.asarray(k.getAccepts(), dtype=np.int64)
        tot = self.sum_counts(np.array([acc.sum(), k.getMovesPerRun() * acc.size]))
        out["accepts"] = int(tot[0])
        out["moves"] = int(tot[1])
        out["acceptance_rate"] = float(tot[0]) / float(tot[1]) if tot[1] else 0.0
        return out
