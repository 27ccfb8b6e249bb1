"""Global-path sweep, precision-study accumulators and the FP64-everywhere arm on the GPU.

* global-path mode (paths in device memory) gives bit-identical results to the shared-
  memory sweep (IEEE build: same operations, same order);
* the FP64-everywhere sweep of a 10-atom LM2M2 cluster agrees with the CPU oracle's FP64
  build (same generator streams; CUDA's and libm's exp/log/sin may differ in the last
  ulp, hence rtol 1e-9 on paths);
* study accumulation: its FP64 column equals the FP64 mode's sums (with float-float
  correlator partials) bit for bit, the device-side correlator moments equal the host
  reduction;
* a small precision study: FP32-path results within statistical error of FP64-everywhere.
"""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()
    engine()


def _cluster(n):
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    return Lm2m2Cluster(n, 1.0)


def _kernel(sysm, walkers, N, S, global_path, double=False, accumulation="fp64", fast=False, op_runs=2,
            msteps=2, ranlux=False, seed=3, partials="fp32"):
    kernel, kernel_args = engine()
    from feynsimul_gb300.precision import hyperradius2
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=walkers, N=N, beta=sysm.beta, S=S, enableOperator=True,
        enableCorrelator=True, enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
        enableBins=False, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True,
        enableGlobalPath=global_path, enableGlobalOldPath=False, enableDouble=double,
        enableRanlux=ranlux, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
        operators=(sysm.energyOp,), correlators=(hyperradius2(sysm.DOF),), operatorRuns=op_runs,
        metroStepsPerOperatorRun=msteps, accumulation=accumulation, fastMath=fast, seed=seed,
        partials=partials)
    k = kernel.PIMCKernel(ka)
    if ranlux:
        k.initRanlux()
        k.groupInitRanlux()
    return k


@pytest.mark.parametrize("ranlux", [False, True], ids=["xorshift", "ranlux"])
def test_global_path_bit_identical_to_shared(ranlux):
    sysm = _cluster(3)
    ks = _kernel(sysm, 64, 64, 3, False, ranlux=ranlux)
    kg = _kernel(sysm, 64, 64, 3, True, ranlux=ranlux)
    p0 = sysm.initial_paths(64, 64, np.random.RandomState(1)).astype(np.float32)
    for k in (ks, kg):
        k.setPaths(p0)
    if ranlux:
        kg.setRanluxTables(*ks.getRanluxTables())
    else:
        kg.setSeeds(ks.getSeeds())
        kg.setWalkerSeeds(ks.getWalkerSeeds())
    for _ in range(3):
        ks.run()
        kg.run()
    assert np.array_equal(ks.getPaths(), kg.getPaths())
    assert np.array_equal(ks.getAccepts(), kg.getAccepts())
    assert np.array_equal(ks._raw_operators(), kg._raw_operators())
    assert np.array_equal(ks._raw_correlator(), kg._raw_correlator())
    ks.close()
    kg.close()


def test_fp64_everywhere_matches_oracle():
    from oracle.oracle import OracleConfig, OracleSampler
    from feynsimul_gb300.precision import hyperradius2
    sysm = _cluster(10)
    W, N, S = 4, 32, 2
    k = _kernel(sysm, W, N, S, True, double=True, fast=False, op_runs=2, msteps=2)
    o = OracleSampler(OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=W, N=N, beta=sysm.beta,
        S=S, operatorRuns=2, metroStepsPerOperatorRun=2, enableDouble=True, operators=(sysm.energyOp,),
        correlators=(hyperradius2(sysm.DOF),), accum=1))
    p0 = sysm.initial_paths(W, N, np.random.RandomState(2), noise=0.02)
    k.setPaths(p0)
    o.paths[...] = p0
    o.seeds[...] = k.getSeeds()
    o.walker_seeds[...] = k.getWalkerSeeds()
    for _ in range(2):
        k.run()
        o.run()
        assert np.array_equal(k.getSeeds(), o.seeds)
        assert np.array_equal(k.getAccepts(), o.accepts)
        np.testing.assert_allclose(k.getPaths(), o.paths, rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(k._raw_operators(), o.op_means.reshape(-1), rtol=1e-9)
        np.testing.assert_allclose(k._raw_correlator(), o.cor_means.reshape(-1), rtol=1e-9)
    assert k.getAccepts().sum() > 0
    k.close()


def test_study_columns_and_device_moments():
    sysm = _cluster(4)
    W, N, S = 96, 64, 2
    # IEEE builds: with FMA contraction allowed, two differently generated modules may
    # round the operator expression differently
    ks = _kernel(sysm, W, N, S, True, accumulation="study", fast=False)
    # the study's FP64 column sums each measurement in float-float
    kd = _kernel(sysm, W, N, S, True, accumulation="fp64", fast=False, partials="exact")
    p0 = sysm.initial_paths(W, N, np.random.RandomState(4)).astype(np.float32)
    for k in (ks, kd):
        k.setPaths(p0)
    kd.setSeeds(ks.getSeeds())
    kd.setWalkerSeeds(ks.getWalkerSeeds())
    for _ in range(4):
        ks.run()
        kd.run()
    assert np.array_equal(ks.getPaths(), kd.getPaths())
    raw = ks._raw_correlator().reshape(-1, 4)
    assert np.array_equal(raw[:, 3], kd._raw_correlator())
    np.testing.assert_allclose(raw[:, 0], raw[:, 3], rtol=1e-4)
    np.testing.assert_allclose(raw[:, 1], raw[:, 3], rtol=1e-5)
    st = ks.getOperatorsStudy()
    np.testing.assert_allclose(st[2], kd.getOperators(), rtol=1e-14)  # host vs device mean
    np.testing.assert_allclose(st[0], st[2], rtol=1e-5)
    # device moments vs the host reduction of the per-walker values
    per = ks.getCorrelatorStudy()                       # (3, W, 1, N/2)
    m, se = ks.getCorrelatorMoments()
    np.testing.assert_allclose(m, per.mean(axis=1), rtol=1e-12)
    np.testing.assert_allclose(se, per.std(axis=1) / np.sqrt(W), rtol=1e-6)
    m2, _ = ks.getCorrelatorMoments((10, 50))
    np.testing.assert_allclose(m2, per[:, 10:50].mean(axis=1), rtol=1e-12)
    mean, _ = kd.getCorrelator()
    md, _ = kd.getCorrelatorMoments()
    np.testing.assert_allclose(md, mean, rtol=1e-12)
    ks.close()
    kd.close()


def test_set_paths_tiled():
    sysm = _cluster(3)
    k = _kernel(sysm, 100, 32, 2, True)
    t = np.random.RandomState(0).randn(7, sysm.DOF * 32).astype(np.float32)
    with pytest.raises(Exception):
        k.setPathsTiled(t[:, :5])
    k.setPathsTiled(t)
    got = k.getPaths()
    assert np.array_equal(got, t[np.arange(100) % 7])
    k.close()


def test_small_precision_study():
    from feynsimul_gb300.precision import precision_study
    r = precision_study(n_atoms=4, N=64, walkers=8192, S=3, op_runs=4, msteps=2, launches=4,
                        fp64_walkers=2048, n_templates=64, seed=5)
    e, c = r["energy"], r["correlator_rho2"]
    print(r)
    # the FP32-path result lies within its statistical error of FP64 everywhere (the paired
    # difference, which resolves the systematic FP32 arithmetic error, is reported only)
    assert abs(e["z_unpaired"]) < 4, e
    assert e["diff_rel"] < 1e-2, e
    assert c["max_abs_z_over_lags"] < 5, c
    assert e["fp32_sum_rel_err"] < 1e-5 and e["kahan_sum_rel_err"] <= e["fp32_sum_rel_err"] + 1e-9
    assert c["kahan_sum_rel_err_max_over_lags"] <= c["fp32_sum_rel_err_max_over_lags"] + 1e-9
    assert 0.05 < r["acceptance_fp32"] < 1 and 0.05 < r["acceptance_fp64"] < 1
