"""Physics on the GPU: exact discretised harmonic oscillator values, the run loop, and
bit-identical resume from a checkpoint."""
import types

import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


def exact_ho(beta, N, taus):
    """Primitive-action HO (m = omega = hbar = 1), N periodic slices: the path is Gaussian with
    precision matrix (2 - shift - shift^T)/eps + eps; its eigenvalues are
    lambda_k = (2 - 2 cos(2 pi k / N)) / eps + eps.  <x^2> = mean(1/lambda) and
    C(tau) = mean(cos(2 pi k tau / N) / lambda).  The virial energy of V = x^2/2 is <x^2>."""
    eps = beta / N
    k = np.arange(N)
    lam = (2 - 2 * np.cos(2 * np.pi * k / N)) / eps + eps
    return np.mean(1 / lam), np.array([np.mean(np.cos(2 * np.pi * k * t / N) / lam) for t in taus])


def _ho_kernel(N=64, S=3, walkers=2048, beta=8.0, op_runs=40, msteps=2, ranlux=False, **extra):
    kernel, kernel_args = engine()
    sysm = types.SimpleNamespace(DOF=1, potential="0.5 * 1.0 * x1 * x1",
                                 userCode="FLOAT_TYPE sqr(FLOAT_TYPE x){return x*x;}")
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=walkers, N=N, beta=beta, S=S, enableOperator=True,
        enableCorrelator=True, enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
        enableBins=extra.pop("enableBins", False), nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True,
        enableGlobalPath=False, enableGlobalOldPath=False, enableRanlux=ranlux, luxuaryFactor=2,
        ranluxIntMax=2 ** 32 - 1, operators=("1.0 * x1 * x1",), correlators=("x1",), operatorRuns=op_runs,
        metroStepsPerOperatorRun=msteps, seed=7, **extra)
    k = kernel.PIMCKernel(ka)
    if ranlux:
        k.initRanlux()
        k.groupInitRanlux()
    return k


@pytest.mark.parametrize("ranlux", [False, True])
def test_ho_matches_exact_discretised_values(ranlux):
    require_gpu()
    N, beta = 64, 8.0
    k = _ho_kernel(N=N, beta=beta, ranlux=ranlux)
    for _ in range(5):  # burn-in from the straight x=0 paths
        k.run()
    k.zeroAccumulators()
    e = []
    for _ in range(20):
        k.run()
        e.append(k.getOperators()[0].mean())
    e = np.array(e)
    x2, c = exact_ho(beta, N, range(N // 2))
    # runs are separated by 80 sweeps; treat them as independent batch means
    se = e.std(ddof=1) / np.sqrt(len(e))
    assert abs(e.mean() - x2) < 5 * se + 1e-4, (e.mean(), x2, se)
    mean, stderr = k.getCorrelator()
    # correlator: each walker's mean over the 20 runs; the walkers are independent chains,
    # so the per-walker spread / sqrt(walkers) is the standard error of the ensemble mean
    m2, se2 = k.getCorrelatorMoments()
    np.testing.assert_allclose(m2, mean, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(se2, stderr, rtol=1e-6, atol=1e-12)
    tol = 5 * stderr[0, :8] + 1e-5
    # the tolerance must resolve the values it checks: well below C(tau) itself
    assert np.all(tol < 0.05 * np.abs(c[:8])), (tol, c[:8])
    assert np.all(np.abs(mean[0, :8] - c[:8]) < tol), (mean[0, :8], c[:8], stderr[0, :8])
    k.close()


def test_ho_bins_follow_the_exact_gaussian():
    """Known answer |psi_0|^2 (the reference tutorial's density plot): the discretised HO's
    path marginal is exactly Gaussian with variance <x^2> = mean(1/lambda_k), so the bin
    density (kernel.c:478-507, kernel.py:619-637) must follow N(0, <x^2>) averaged over each
    bin; at beta = 8 that is the ground state's exp(-x^2)/sqrt(pi) to 0.1%."""
    import math
    require_gpu()
    N, beta, lo, hi, nb = 64, 8.0, -3.0, 3.0, 30
    k = _ho_kernel(N=N, beta=beta, enableBins=True, xMin=lo, xMax=hi, binResolutionPerDOF=nb)
    for _ in range(5):
        k.run()
    k.zeroAccumulators()
    for _ in range(10):
        k.run()
    d = k.getBinCounts()
    assert d.shape == (nb,)
    x2, _ = exact_ho(beta, N, [])
    edges = np.linspace(lo, hi, nb + 1)
    cdf = np.array([0.5 * (1.0 + math.erf(e / math.sqrt(2.0 * x2))) for e in edges])
    want = np.diff(cdf) / np.diff(edges)
    assert np.all(np.abs(d - want) < 5e-3 + 0.02 * want), np.abs(d - want).max()
    assert abs(d.sum() * (hi - lo) / nb - (cdf[-1] - cdf[0])) < 2e-3
    k.close()


def test_checkpoint_resume_is_bit_identical(tmp_path):
    require_gpu()
    a = _ho_kernel(walkers=256)
    for _ in range(4):
        a.run()
    b = _ho_kernel(walkers=256)
    for _ in range(2):
        b.run()
    b.saveCheckpoint(str(tmp_path / "ck.npz"))
    b.close()
    c = _ho_kernel(walkers=256)
    c.loadCheckpoint(str(tmp_path / "ck.npz"))
    for _ in range(2):
        c.run()
    sa, sc = a.getState(), c.getState()
    for key in ("paths", "seeds", "walker_seeds", "correlator"):
        assert np.array_equal(sa[key], sc[key]), key
    np.testing.assert_array_equal(a.getOperators(), c.getOperators())
    a.close()
    c.close()


def test_modn_short_run(tmp_path):
    require_gpu()
    _, kernel_args = engine()
    from feynsimul_gb300.pimc_utils import modN, read_tsv
    from feynsimul_gb300.physical_systems.harm_osc import HarmOsc
    sysm = HarmOsc()
    ka = kernel_args.KernelArgs(
        nbrOfWalkers=64, N=8, enablePathShift=False, enableBisection=True, enableSingleNodeMove=False,
        enableGlobalPath=True, enableGlobalOldPath=True, enableParallelizePath=True, enableBins=False,
        beta=20.0, nbrOfWalkersPerWorkGroup=4, operatorRuns=300, enableOperator=True,
        enableCorrelator=False, metroStepsPerOperatorRun=40, system=sysm, operators=(sysm.energyOp,))
    start = np.random.RandomState(0).uniform(size=(64, 1), low=-1.0, high=1.0) * 0.01
    modN(ka, start, 3, "SHO", lambda N, S: max(2 ** 6 // 2 ** S, 1), lambda N, S: 4,
         lambda N, S: 3, 512, finalN=32, simTime=0, resultsDir=str(tmp_path), checkpointEvery=2)
    import glob
    tsv = glob.glob(str(tmp_path / "SHO" / "*" / "*" / "data.tsv"))
    assert len(tsv) == 1
    beta, rows, ops = read_tsv(tsv[0])
    assert beta == 20.0
    Ns = [r[0] for r in rows]
    assert Ns[:3] == [8, 8, 8] and Ns[3:6] == [16, 16, 16] and Ns[6:9] == [32, 32, 32]
    assert ops.shape[1:] == (1, 64)
    # energies rise towards 0.5 with N (the reference tutorial shows 0.31 -> 0.42 -> 0.49)
    e8, e32 = ops[:3].mean(), ops[6:9].mean()
    assert e8 < e32 < 0.55
    outdir = tsv[0].rsplit("/", 1)[0]
    assert glob.glob(outdir + "/pathsN32episode*") and glob.glob(outdir + "/checkpoint.npz")


def _ho_walker_kernel(moves, walkers=2048, N=16, beta=4.0, op_runs=50, msteps=4, seed=9):
    kernel, kernel_args = engine()
    sysm = types.SimpleNamespace(DOF=1, potential="0.5 * 1.0 * x1 * x1", userCode="")
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=walkers, N=N, beta=beta, S=2, enableOperator=True, enableCorrelator=False,
        enableBisection="bisection" in moves, enablePathShift="shift" in moves,
        enableSingleNodeMove="single" in moves, alpha=0.8, PSAlpha=0.5, enableBins=False,
        nbrOfWalkersPerWorkGroup=1, enableParallelizePath=False, enableGlobalPath=False,
        enableGlobalOldPath=False, operators=("1.0 * x1 * x1",), operatorRuns=op_runs,
        metroStepsPerOperatorRun=msteps, seed=seed)
    return kernel.PIMCKernel(ka)


@pytest.mark.parametrize("moves", [("single",), ("shift", "single"), ("shift", "bisection")])
def test_ho_walker_moves_match_exact_values(moves):
    """Single-node and path-shift moves (kernel.c:640-705) sample the exact discretised HO.
    The fixed mode carries the single-node counter across launches, so every node moves."""
    require_gpu()
    N, beta = 16, 4.0
    k = _ho_walker_kernel(moves, N=N, beta=beta)
    for _ in range(10):
        k.run()
    e = []
    for _ in range(30):
        k.run()
        e.append(k.getOperators()[0].mean())
    e = np.array(e)
    x2, _ = exact_ho(beta, N, [0])
    tau_guard = 3.0  # launches are correlated for local moves: widen the error bar
    se = e.std(ddof=1) / np.sqrt(len(e)) * tau_guard
    assert abs(e.mean() - x2) < 5 * se + 2e-3, (e.mean(), x2, se)
    assert 0.1 < k.getAcceptanceRate() < 1.0
    k.close()


def test_walker_moves_checkpoint_resume_is_bit_identical(tmp_path):
    """Resuming restores the move counter too: the continued run equals the unbroken one."""
    require_gpu()
    mv = ("shift", "single", "bisection")
    a = _ho_walker_kernel(mv, walkers=128, op_runs=3, msteps=5)
    for _ in range(4):
        a.run()
    b = _ho_walker_kernel(mv, walkers=128, op_runs=3, msteps=5)
    for _ in range(2):
        b.run()
    b.saveCheckpoint(str(tmp_path / "ck.npz"))
    b.close()
    c = _ho_walker_kernel(mv, walkers=128, op_runs=3, msteps=5)
    c.loadCheckpoint(str(tmp_path / "ck.npz"))
    for _ in range(2):
        c.run()
    sa, sc = a.getState(), c.getState()
    for key in ("paths", "seeds", "walker_seeds", "step_counter"):
        assert np.array_equal(sa[key], sc[key]), key
    np.testing.assert_array_equal(a.getAccepts(), c.getAccepts())
    a.close()
    c.close()
