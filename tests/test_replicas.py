"""Multi-GPU replicas, host side, as two gloo ranks on the CPU: distinct per-rank seeds, the
ensemble merge of the FP64 accumulators and the max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_values(rank):
    return np.random.RandomState(100 + rank).randn(1000 + 37 * rank) * (1 + rank) + rank


class _FakeKernel:
    """The getters of a PIMCKernel that ReplicaGroup.merge_kernel reads, with per-rank
    numbers (no GPU): 2 operators, 1 correlator of 4 lags, a 5-bin histogram, 3 bins."""

    _enableOperator = True
    _enableCorrelator = True
    _histBins = 5
    _enableBins = True

    def __init__(self, rank):
        rs = np.random.RandomState(7 + rank)
        self.W = 300 + 50 * rank
        # a large mean and a small spread: a sum of squares of the raw values would cancel
        self.ops = np.stack([1e6 + rs.randn(self.W) * 1e-3, rs.randn(self.W) + rank])
        self.cor = rs.rand(self.W, 1, 4) + rank
        self.hist = np.arange(5, dtype=np.uint64) * (rank + 1) + 2 ** 40
        self.bins = np.array([rank, 2, 3], np.uint32)
        self.acc = rs.randint(0, 20, size=4 * self.W).astype(np.uint32)

    def getOperators(self):
        return self.ops

    def getCorrelatorPerWalker(self):
        return self.cor

    def getHistogram(self, density=True):
        return np.arange(5) + 0.5, self.hist

    def getBinCountsRaw(self):
        return self.bins

    def getAccepts(self):
        return self.acc

    def getMovesPerRun(self):
        return 20


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from feynsimul_gb300.replicas import ReplicaGroup, replica_seed
        g = ReplicaGroup()
        assert (g.rank, g.world) == (rank, world)
        merged = g.merge(_rank_values(rank))
        t = g.max(0.5 + rank)
        np.save(os.path.join(out_dir, f"r{rank}.npy"),
                np.array([merged["walkers"], merged["mean"], merged["se"], t, replica_seed(17, rank)]))
        mk = g.merge_kernel(_FakeKernel(rank))
        np.savez(os.path.join(out_dir, f"k{rank}.npz"), op_mean=mk["operators"]["mean"],
                 op_se=mk["operators"]["se"], op_n=mk["operators"]["walkers"],
                 cor_mean=mk["correlator"]["mean"], cor_se=mk["correlator"]["se"],
                 hist=mk["histogram_counts"], bins=mk["bin_counts"], acc=mk["accepts"], moves=mk["moves"])
    finally:
        dist.destroy_process_group()


def test_replica_merge_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f"r{r}.npy") for r in range(world)]
    x = np.concatenate([_rank_values(r) for r in range(world)])
    for r in res:  # every rank holds the same merged estimate
        assert int(r[0]) == x.size
        np.testing.assert_allclose(r[1], x.mean(), rtol=1e-12)
        np.testing.assert_allclose(r[2], x.std() / np.sqrt(x.size), rtol=1e-9)
        assert r[3] == 0.5 + world - 1
    assert res[0][4] != res[1][4]
    # every accumulator of the kernel merged: the same on both ranks, and equal to the
    # pooled walkers' values computed here in one place
    fk = [_FakeKernel(r) for r in range(world)]
    ops = np.concatenate([f.ops for f in fk], axis=1)
    cor = np.concatenate([f.cor for f in fk], axis=0)
    ks = [np.load(tmp_path / f"k{r}.npz") for r in range(world)]
    for k in ks:
        assert int(k["op_n"]) == ops.shape[1]
        np.testing.assert_allclose(k["op_mean"], ops.mean(axis=1), rtol=1e-14)
        np.testing.assert_allclose(k["op_se"], ops.std(axis=1) / np.sqrt(ops.shape[1]), rtol=1e-9)
        assert k["op_se"][0] > 0          # no cancellation at mean 1e6, spread 1e-3
        np.testing.assert_allclose(k["cor_mean"], cor.mean(axis=0), rtol=1e-13)
        np.testing.assert_allclose(k["cor_se"], cor.std(axis=0) / np.sqrt(cor.shape[0]), rtol=1e-9)
        assert np.array_equal(k["hist"], sum(f.hist.astype(np.int64) for f in fk))
        assert np.array_equal(k["bins"], sum(f.bins.astype(np.int64) for f in fk))
        assert int(k["acc"]) == sum(int(f.acc.sum()) for f in fk)
        assert int(k["moves"]) == sum(20 * f.acc.size for f in fk)
    for name in ks[0].files:
        assert np.array_equal(ks[0][name], ks[1][name]), name


def test_single_process_group_is_identity():
    from feynsimul_gb300.replicas import ReplicaGroup, replica_seed
    g = ReplicaGroup()
    assert (g.rank, g.world) == (0, 1)
    x = _rank_values(0)
    m = g.merge(x)
    assert m["walkers"] == x.size and abs(m["mean"] - x.mean()) < 1e-12
    assert g.max(3.0) == 3.0
    assert len({replica_seed(5, r) for r in range(64)}) == 64
