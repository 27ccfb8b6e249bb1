"""The reference-named few-atom plugins (physical_systems/lm2m2_3part.py, lm2m2_4part.py)
swept on the GPU against the CPU oracle with the same plugin strings: FP64 build, IEEE
math, same generator streams, so accept decisions match exactly and the paths, operator
and correlator sums agree to 1e-9 (CUDA's and libm's exp / log / sin may differ in the
last ulp)."""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()
    engine()


def _paths(sysm, n, W, N, rng):
    """W walkers of n atoms 3-5 Angstrom apart, static paths plus a little noise, in the
    plugin's Jacobi coordinates (unit masses, its length unit)."""
    from feynsimul_gb300.physical_systems.lm2m2 import jacobi_matrix
    unit = sysm.xUnit / 1e-10
    J = jacobi_matrix(n, 1.0)[: n - 1]
    out = np.empty((W, sysm.DOF, N))
    for w in range(W):
        r = rng.normal(0.0, 1.0, size=(n, 3))
        r *= rng.uniform(3.0, 5.0) / min(np.linalg.norm(r[a] - r[b]) for a in range(n) for b in range(a + 1, n))
        xi = (J @ r).reshape(-1) / unit
        out[w] = xi[:, None] + rng.normal(0.0, 0.02, size=(sysm.DOF, N))
    return out.reshape(W, sysm.DOF * N)


@pytest.mark.parametrize("module,cls,n", [("lm2m2_3part", "Lm2m2_3part", 3), ("lm2m2_4part", "Lm2m2_4part", 4)])
def test_few_atom_plugin_sweep_matches_oracle(module, cls, n):
    import importlib
    from oracle.oracle import OracleConfig, OracleSampler
    kernel, kernel_args = engine()
    sysm = getattr(importlib.import_module(f"feynsimul_gb300.physical_systems.{module}"), cls)()
    W, N, S, beta = 8, 32, 2, 200.0
    ops = (sysm.energyOp, sysm.meanSquaredRadiusOp, sysm.meanRadiusOp, sysm.meanSquaredAtomDistOp)
    cors = (sysm.meanSquaredRadiusOp,)
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=W, N=N, beta=beta, S=S, enableOperator=True, enableCorrelator=True,
        enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
        nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
        enableGlobalOldPath=False, enableDouble=True, enableRanlux=False, operators=ops, correlators=cors,
        operatorRuns=2, metroStepsPerOperatorRun=2, accumulation="fp64", fastMath=False, seed=11)
    k = kernel.PIMCKernel(ka)
    o = OracleSampler(OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=W, N=N, beta=beta, S=S,
        operatorRuns=2, metroStepsPerOperatorRun=2, enableDouble=True, operators=ops, correlators=cors, accum=1))
    p0 = _paths(sysm, n, W, N, np.random.RandomState(5))
    k.setPaths(p0)
    o.paths[...] = p0
    o.seeds[...] = k.getSeeds()
    o.walker_seeds[...] = k.getWalkerSeeds()
    for _ in range(2):
        k.run()
        o.run()
        assert np.array_equal(k.getAccepts(), o.accepts)
        np.testing.assert_allclose(k.getPaths(), o.paths, rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(k._raw_operators(), o.op_means.reshape(-1), rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(k._raw_correlator(), o.cor_means.reshape(-1), rtol=1e-9)
    assert 0 < k.getAccepts().sum()
    assert np.all(np.isfinite(k.getOperators()))
    k.close()


def test_three_particle_example_through_modN(tmp_path):
    """The reference's examples/lm2m2_3particles.py set-up (its KernelArgs, plugin and
    operators) driven through modN for a few short episodes: the files appear and the
    energies are finite."""
    import glob
    from feynsimul_gb300.pimc_utils import KernelArgs, modN, read_tsv
    from feynsimul_gb300.physical_systems.lm2m2_3part import Lm2m2_3part
    ka = KernelArgs(nbrOfWalkers=64, N=8, enablePathShift=False, enableBisection=True, enableSingleNodeMove=False,
                    enableGlobalPath=True, enableGlobalOldPath=True, enableParallelizePath=True, enableBins=False,
                    enableDouble=False, enableRanlux=False, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1, beta=1000.0,
                    nbrOfWalkersPerWorkGroup=4, operatorRuns=100, enableOperator=True, enableCorrelator=False,
                    metroStepsPerOperatorRun=40, system=Lm2m2_3part())
    ka.operators = (ka.system.energyOp, ka.system.meanSquaredRadiusOp, ka.system.meanRadiusOp)
    start = np.random.RandomState(1).uniform(size=(ka.nbrOfWalkers, ka.system.DOF), low=-1.0, high=1.0) * 0.01
    modN(ka, start, 3000, "lm2m2_3part", lambda N, S: max(2 ** 6 // 2 ** S, 1), lambda N, S: 4,
         lambda N, S: 2, 512, finalN=16, simTime=0, resultsDir=str(tmp_path))
    tsv = glob.glob(str(tmp_path / "lm2m2_3part" / "*" / "*" / "data.tsv"))
    assert len(tsv) == 1
    beta, rows, ops = read_tsv(tsv[0])
    assert beta == 1000.0 and [r[0] for r in rows] == [8, 8, 16, 16]
    assert ops.shape[1:] == (3, 64) and np.all(np.isfinite(ops))
