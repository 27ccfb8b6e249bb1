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


def test_single_process_group_is_identity():
    from feynsimul_gb300.replicas import ReplicaGroup, replica_seed
    g = ReplicaGroup()
    assert (g.rank, g.world) == (0, 1)
    x = _rank_values(0)
    m = g.merge(x)
    assert m["walkers"] == x.size and abs(m["mean"] - x.mean()) < 1e-12
    assert g.max(3.0) == 3.0
    assert len({replica_seed(5, r) for r in range(64)}) == 64
