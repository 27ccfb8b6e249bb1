"""Ragged batch on the GPU: every system of a batch evolves exactly as the single-system
sweep with the same seeds and paths (fixed-mode xorshift, fast math, FP64 sums)."""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


def test_batch_matches_single_system_kernels():
    require_gpu()
    kernel, kernel_args = engine()
    from feynsimul_gb300.batch import BatchSampler
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    workload = [{"n": 3, "N": 64, "T": 1.0, "walkers": 96}, {"n": 4, "N": 128, "T": 0.7, "walkers": 64},
                {"n": 3, "N": 256, "T": 1.7, "walkers": 32}, {"n": 5, "N": 64, "T": 1.2, "walkers": 64}]
    op_runs, msteps = 2, 3
    b = BatchSampler(workload, op_runs=op_runs, msteps=msteps, block_threads=256, tpw_target=16)
    rng = np.random.RandomState(5)
    singles = []
    for i, w in enumerate(workload):
        c = Lm2m2Cluster(w["n"], w["T"])
        S = b.systems[i].bisection_level
        tpw = w["N"] >> S
        paths = c.initial_paths(w["walkers"], w["N"], rng).astype(np.float32)
        ts = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"] * tpw + 1, 4)).astype(np.uint32)
        ws = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"], 4)).astype(np.uint32)
        b.set_state(i, paths, ts[:-1], ws)
        ka = kernel_args.KernelArgs(
            system=c, nbrOfWalkers=w["walkers"], N=w["N"], beta=float(1.0 / w["T"]), S=S, enableOperator=True,
            enableCorrelator=False, enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
            enableBins=False, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
            enableGlobalOldPath=False, operators=(c.energyOp,), operatorRuns=op_runs,
            metroStepsPerOperatorRun=msteps, fastMath=True, accumulation="fp64")
        k = kernel.PIMCKernel(ka)
        k.setPaths(paths)
        k.setSeeds(ts)
        k.setWalkerSeeds(ws)
        singles.append(k)
    b.run(1, graph=True)
    for i, (w, k) in enumerate(zip(workload, singles)):
        k.run()
        acc_b, acc_s = b.accepts(i), k.getAccepts()
        same = np.all(np.isclose(b.paths(i), k.getPaths(), rtol=1e-4, atol=1e-4), axis=1)
        assert same.mean() > 0.95, (i, same.mean())
        assert (acc_b != acc_s).sum() <= max(2, acc_s.size // 100), i
        # per-walker energy: batch keeps sums over (runs x slices), the kernel per-walker means
        e_b = b.energy_sums(i) / (op_runs * w["N"])
        e_s = k.getOperators()[0]
        np.testing.assert_allclose(e_b[same], e_s[same], rtol=1e-3, atol=1e-3)
        k.close()
    # a second launch through the captured graph continues the same chains
    t = b.run(2, graph=True)
    assert t > 0
    b.close()


def test_autotune_caches(tmp_path):
    require_gpu()
    engine()
    from feynsimul_gb300.batch import autotune, ragged_workload
    wl = ragged_workload(seed=3, n_systems=6, walker_range=(64, 256))
    cache = str(tmp_path / "tune.json")
    r1 = autotune(wl, candidates=[(256, 16), (128, 16)], cache_file=cache, launches=1)
    assert not r1["cached"] and r1["node_updates_per_s"] > 0
    r2 = autotune(wl, candidates=[(256, 16), (128, 16)], cache_file=cache, launches=1)
    assert r2["cached"] and r2["block_threads"] == r1["block_threads"]


def test_batch_systems_match_oracle():
    """Every system of a small ragged batch (3-6 atoms, different N, T, walker counts and
    bisection levels) against the oracle run on that system alone with the same paths and
    xorshift rows (fixed mode).  The batch computes in fast math (__logf, __sinf, __expf)
    and the oracle with the C library, so a few accept decisions may flip; walkers none of
    whose work-items flipped must keep the oracle's paths and per-walker energies."""
    require_gpu()
    engine()
    from feynsimul_gb300.batch import BatchSampler
    from oracle.oracle import OracleConfig, OracleSampler
    workload = [{"n": 3, "N": 64, "T": 1.0, "walkers": 64}, {"n": 4, "N": 128, "T": 0.7, "walkers": 32},
                {"n": 5, "N": 64, "T": 1.5, "walkers": 32}, {"n": 6, "N": 32, "T": 0.6, "walkers": 32},
                {"n": 3, "N": 256, "T": 1.8, "walkers": 32}]
    op_runs, msteps = 2, 3
    b = BatchSampler(workload, op_runs=op_runs, msteps=msteps, block_threads=256, tpw_target=16)
    rng = np.random.RandomState(8)
    oracles = []
    for i, w in enumerate(workload):
        c = b.clusters[w["n"]]
        S = b.systems[i].bisection_level
        tpw = w["N"] >> S
        paths = c.initial_paths(w["walkers"], w["N"], rng).astype(np.float32)
        ts = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"] * tpw + 1, 4)).astype(np.uint32)
        ws = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"], 4)).astype(np.uint32)
        b.set_state(i, paths, ts[:-1], ws)
        o = OracleSampler(OracleConfig(
            DOF=c.DOF, potential=c.potential, userCode=c.userCode, nbrOfWalkers=w["walkers"], N=w["N"],
            beta=float(1.0 / w["T"]), S=S, operatorRuns=op_runs, metroStepsPerOperatorRun=msteps,
            operators=(c.energyOp,), compat=False, accum=1))
        o.paths[...] = paths
        o.seeds[...] = ts
        o.walker_seeds[...] = ws
        oracles.append(o)
    b.run(1, graph=False)
    for i, (w, o) in enumerate(zip(workload, oracles)):
        o.run()
        tpw = w["N"] >> b.systems[i].bisection_level
        diff = b.accepts(i) != o.accepts
        assert diff.mean() <= 0.05, (i, diff.mean())
        keep = ~diff.reshape(w["walkers"], tpw).any(axis=1)
        assert keep.mean() >= 0.5, (i, keep.mean())
        np.testing.assert_allclose(b.paths(i)[keep], o.paths[keep], rtol=2e-3, atol=2e-4)
        e_b = b.energy_sums(i) / (op_runs * w["N"])
        e_o = o.op_means.reshape(w["walkers"], tpw).mean(axis=1)
        np.testing.assert_allclose(e_b[keep], e_o[keep], rtol=2e-3, atol=2e-3)
    b.close()


def test_batch_systems_match_oracle_ranlux():
    """The same per-system check with RANLUX streams (luxury 2, the kernel's 3: p = 224):
    every system's tables after the launch equal the oracle's bit for bit (a move draws the
    same count of numbers whatever its decision), and the accepts, paths and energies agree
    as in the xorshift case."""
    require_gpu()
    engine()
    from feynsimul_gb300.batch import BatchSampler
    from oracle.oracle import OracleConfig, OracleSampler
    workload = [{"n": 3, "N": 64, "T": 1.0, "walkers": 64}, {"n": 4, "N": 128, "T": 0.7, "walkers": 32},
                {"n": 5, "N": 64, "T": 1.5, "walkers": 32}, {"n": 6, "N": 32, "T": 0.6, "walkers": 32}]
    op_runs, msteps = 2, 3
    b = BatchSampler(workload, op_runs=op_runs, msteps=msteps, block_threads=256, tpw_target=16, ranlux=2)
    rng = np.random.RandomState(9)
    oracles = []
    for i, w in enumerate(workload):
        c = b.clusters[w["n"]]
        S = b.systems[i].bisection_level
        tpw = w["N"] >> S
        paths = c.initial_paths(w["walkers"], w["N"], rng).astype(np.float32)
        ts = np.zeros((w["walkers"] * tpw, 4), np.uint32)
        ws = np.zeros((w["walkers"], 4), np.uint32)
        b.set_state(i, paths, ts, ws)  # the paths; the xorshift rows are unused here
        t, g = b.ranlux_tables(i)
        assert len({row.tobytes() for row in t}) == t.shape[0]  # distinct per thread
        o = OracleSampler(OracleConfig(
            DOF=c.DOF, potential=c.potential, userCode=c.userCode, nbrOfWalkers=w["walkers"], N=w["N"],
            beta=float(1.0 / w["T"]), S=S, operatorRuns=op_runs, metroStepsPerOperatorRun=msteps,
            enableRanlux=True, luxuaryFactor=2, operators=(c.energyOp,), compat=False, accum=1))
        o.paths[...] = paths
        o.ranlux_tab[...] = t
        o.group_tab[...] = g
        oracles.append(o)
    b.run(1, graph=False)
    for i, (w, o) in enumerate(zip(workload, oracles)):
        o.run()
        t, g = b.ranlux_tables(i)
        assert np.array_equal(t, o.ranlux_tab), i
        assert np.array_equal(g, o.group_tab), i
        tpw = w["N"] >> b.systems[i].bisection_level
        diff = b.accepts(i) != o.accepts
        assert diff.mean() <= 0.05, (i, diff.mean())
        keep = ~diff.reshape(w["walkers"], tpw).any(axis=1)
        assert keep.mean() >= 0.5, (i, keep.mean())
        np.testing.assert_allclose(b.paths(i)[keep], o.paths[keep], rtol=2e-3, atol=2e-4)
        e_b = b.energy_sums(i) / (op_runs * w["N"])
        e_o = o.op_means.reshape(w["walkers"], tpw).mean(axis=1)
        np.testing.assert_allclose(e_b[keep], e_o[keep], rtol=2e-3, atol=2e-3)
    b.close()
