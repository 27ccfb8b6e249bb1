"""Parity of the benchmarked configuration: three He-4 atoms with the LM2M2 potential
(Lm2m2Cluster(3, 1.0), T = 1 K), N = 256 slices, bisection level S = 4, RANLUX
(luxuaryFactor 2, fixed mode), FP32 paths, FP64 operator sums, the virial energy
(lm2m2_cluster.py:75-76) and the 200-bin pair-distance histogram on 0-20 Angstrom --
the sweep bench.py times -- against the oracle (oracle/pimc_oracle.c).

(a) IEEE math (fastMath=False), 32 walkers, 2 launches, the oracle's FP32 build on the same
    RANLUX tables: tables bit-exact after every launch, at most one accept decision flipped
    (CUDA's and the C library's log / sin / exp / rsqrt may round differently in the last
    ulp), and without a flip paths (rtol 1e-4), energy sums (rtol 1e-4, atol 1e-4 K: the
    virial energy cancels pair terms of tens of Kelvin) and histogram counts equal to the
    oracle's (counts: a pair distance within an ulp of a bin edge may change bin).
(b) The benchmarked code itself (fastMath=True: __logf / __sinf / __expf), 2048 walkers, one
    launch on the same tables as the oracle's FP32 build: tables still bit-exact, and the
    fraction of work-items whose accept count differs is reported and bounded.
(c) Ensemble agreement with the oracle's FP64 build (paths, action, potential and sums in
    FP64, its own FP64 RANLUX streams, so a statistically independent run from the same
    starting paths): 16 groups x 128 walkers on each side, the same number of sweeps.  The
    ensemble virial energy must agree within 3 standard errors (errors from the spread over
    the independent walkers), and the pair-distance histogram passes a chi-square test over
    its populated bins, with per-bin errors from the spread over the 16 independent groups.
    At T = 1 K the trimer is not bound (its ground state is -0.126 K), so the ensemble drifts
    apart; both sides start from the same walkers and make the same number of sweeps, so
    their distributions at equal Monte Carlo time still agree.
(d) The same ensemble check on a bound case: the reference's three-particle example
    (examples/lm2m2_3particles.py:32-77: Lm2m2_3part, beta = 1000, global paths, 4 walkers
    per work group, xorshift), here at N = 16, S = 2, 16 groups x 64 walkers, all three of
    its operators (energy, mean squared radius, mean radius).
"""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu

HIST = dict(histRange=(0.0, 20.0), histBins=200)


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()
    engine()


def _he3():
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    return Lm2m2Cluster(3, 1.0)


def _he3_ka(sysm, walkers, op_runs, msteps, lux=2):
    return dict(nbrOfWalkers=walkers, N=256, beta=float(sysm.beta), S=4, enableOperator=True,
                enableCorrelator=False, enableBisection=True, enablePathShift=False,
                enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
                enableParallelizePath=True, enableGlobalPath=False, enableGlobalOldPath=False,
                enableDouble=False, enableRanlux=True, luxuaryFactor=lux, ranluxIntMax=2 ** 32 - 1,
                operators=(sysm.energyOp,), operatorRuns=op_runs, metroStepsPerOperatorRun=msteps)


def _gpu_kernel(sysm, ka, seed, fast, hist=True):
    kernel, kernel_args = engine()
    extra = dict(histograms=sysm.pairDistanceOps, **HIST) if hist else {}
    k = kernel.PIMCKernel(kernel_args.KernelArgs(system=sysm, seed=seed, fastMath=fast, **extra, **ka))
    if ka["enableRanlux"]:
        k.initRanlux()
        k.groupInitRanlux()
    return k


def _oracle(sysm, ka, double, hist=True, accum=1):
    from oracle.oracle import OracleConfig, OracleSampler
    return OracleSampler(OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=ka["nbrOfWalkers"],
        N=ka["N"], beta=ka["beta"], S=ka["S"], operatorRuns=ka["operatorRuns"],
        metroStepsPerOperatorRun=ka["metroStepsPerOperatorRun"],
        nbrOfWalkersPerWorkGroup=ka["nbrOfWalkersPerWorkGroup"], enableParallelizePath=True,
        enableRanlux=ka["enableRanlux"], luxuaryFactor=ka["luxuaryFactor"], ranluxIntMax=ka["ranluxIntMax"],
        enableDouble=double, operators=tuple(ka["operators"]), compat=False, accum=accum,
        histograms=sysm.pairDistanceOps if hist else (), histRange=HIST["histRange"] if hist else (0.0, 1.0),
        histBins=HIST["histBins"] if hist else 0))


def _oracle_walker_means(o, ka):
    """Per-walker operator means (nOps, walkers) from the oracle's per-work-item FP64 means
    (walker-major work-item ids: one walker per work group here)."""
    nops = len(ka["operators"])
    T = ka["N"] // 2 ** ka["S"]
    per = o.op_means.reshape(ka["nbrOfWalkers"], T, nops)
    return per.mean(axis=1).T


def _same_tables(k, o):
    t, g = k.getRanluxTables()
    o.ranlux_tab[...] = t
    o.group_tab[...] = g


# ------------------------------------------------------------------------- (a)
@pytest.mark.parametrize("lux", [2, 0, 1, 3])
def test_he3_bench_config_ieee_matches_oracle(lux):
    """lux 2 is the benchmarked luxury; 0, 1 and 3 (skips of 24, 76 and 380 steps per 24
    outputs, the first in the per-cycle scheme) take the generator's other branches, whose
    12-value draws of the six-DOF move run as single blocks or as four-value calls."""
    sysm = _he3()
    ka = _he3_ka(sysm, walkers=32, op_runs=2, msteps=5, lux=lux)
    k = _gpu_kernel(sysm, ka, seed=3, fast=False)
    o = _oracle(sysm, ka, double=False)
    p0 = sysm.initial_paths(32, 256, np.random.RandomState(11)).astype(np.float32)
    k.setPaths(p0)
    o.paths[...] = p0
    _same_tables(k, o)
    # the GPU's table seeding equals the oracle's ranluxcl_init of the same rows
    o2 = _oracle(sysm, ka, double=False)
    o2.init_ranlux_rows(o2.ranlux_tab, (np.uint64(int(k._seeds[0])) << np.uint64(32))
                        + np.arange(o2.ranlux_tab.shape[0], dtype=np.uint64))
    assert np.array_equal(o2.ranlux_tab, o.ranlux_tab)
    flips = 0
    for it in range(2):
        k.run()
        o.run()
        t, g = k.getRanluxTables()
        assert np.array_equal(t, o.ranlux_tab)
        assert np.array_equal(g, o.group_tab)
        flips += int((k.getAccepts() != o.accepts).sum())
        assert flips <= 1, flips
        if flips == 0:
            np.testing.assert_allclose(k.getPaths(), o.paths, rtol=1e-4, atol=1e-5)
            # the virial energy is a difference of pair terms of tens of Kelvin (V and
            # r^2 dV/dr^2), so a work-item's sum carries FP32 rounding of about 1e-6 of
            # those terms: absolute tolerance 1e-4 K
            raw = k._raw_operators()
            np.testing.assert_allclose(raw, o.op_means.reshape(-1)[:raw.size], rtol=1e-4, atol=1e-4)
            np.testing.assert_allclose(k.getOperators(), _oracle_walker_means(o, ka), rtol=1e-4, atol=1e-4)
            _, h = k.getHistogram(density=False)
            assert h.sum() == o.hist.sum() or abs(int(h.sum()) - int(o.hist.sum())) <= 4
            assert np.abs(h.astype(np.int64) - o.hist.astype(np.int64)).sum() <= 8
    assert k.getAccepts().sum() > 0
    assert o.hist.sum() > 0.9 * 32 * 256 * 3 * 2 * (it + 1)     # most pair distances inside 0-20 A
    k.close()


# ------------------------------------------------------------------------- (b)
def test_he3_bench_config_fast_math_flip_rate():
    sysm = _he3()
    W = 2048
    ka = _he3_ka(sysm, walkers=W, op_runs=2, msteps=5)
    k = _gpu_kernel(sysm, ka, seed=5, fast=True)
    o = _oracle(sysm, ka, double=False)
    p0 = sysm.initial_paths(W, 256, np.random.RandomState(12)).astype(np.float32)
    k.setPaths(p0)
    o.paths[...] = p0
    _same_tables(k, o)
    k.run()
    o.run()
    t, g = k.getRanluxTables()
    # the generators' consumption does not depend on the accept decisions
    assert np.array_equal(t, o.ranlux_tab)
    assert np.array_equal(g, o.group_tab)
    diff = k.getAccepts() != o.accepts
    rate = float(diff.mean())
    moves = ka["operatorRuns"] * ka["metroStepsPerOperatorRun"]
    print(f"\nfast-math vs IEEE oracle, one launch of {moves} sweeps: {int(diff.sum())} of {diff.size} "
          f"work-items ({100 * rate:.2f} %) differ in their accept count")
    assert rate < 0.10
    # walkers none of whose work-items flipped still follow the oracle closely
    same = ~diff.reshape(W, -1).any(axis=1)
    assert same.sum() > W // 2
    np.testing.assert_allclose(k.getPaths()[same], o.paths[same], rtol=2e-3, atol=2e-4)
    np.testing.assert_allclose(k.getOperators()[:, same], _oracle_walker_means(o, ka)[:, same], rtol=2e-3, atol=1e-4)
    k.close()


# ------------------------------------------------------------------------- (c), (d)
def _ensemble(make_gpu, make_orc, init_paths, groups, burn_launches, launches, nops, hist):
    """Per-walker operator means over the measured launches and per-group histogram counts,
    GPU and oracle, every group from the same starting walkers on both sides."""
    res = {"gpu": {"ops": [], "hist": []}, "orc": {"ops": [], "hist": []}}
    for gi in range(groups):
        p0 = init_paths(gi)
        k = make_gpu(gi)
        o = make_orc(gi)
        k.setPaths(p0.astype(np.float32))
        o.paths[...] = p0
        for _ in range(burn_launches):
            k.run()
            o.run()
        if hist:
            k.zeroAccumulators()
            o.hist[...] = 0
        og, oo = 0.0, 0.0
        for _ in range(launches):
            k.run()
            o.run()
            og = og + k.getOperators()
            oo = oo + o.walker_means()
        res["gpu"]["ops"].append(og / launches)
        res["orc"]["ops"].append(oo / launches)
        if hist:
            res["gpu"]["hist"].append(k.getHistogram(density=False)[1].astype(np.float64))
            res["orc"]["hist"].append(o.hist.astype(np.float64))
        k.close()
    for side in res.values():
        side["ops"] = np.concatenate(side["ops"], axis=1)       # (nOps, walkers)
        if hist:
            side["hist"] = np.stack(side["hist"])               # (groups, bins)
    return res


def _z_operators(res, names):
    out = {}
    for j, name in enumerate(names):
        a, b = res["gpu"]["ops"][j], res["orc"]["ops"][j]
        se = np.sqrt(a.var(ddof=1) / a.size + b.var(ddof=1) / b.size)
        out[name] = ((a.mean() - b.mean()) / se, a.mean(), b.mean(), se)
    return out


def _chi2_hist(res):
    """Chi-square of the difference of the two normalised histograms over the bins both
    populate, per-bin variance from the spread over the independent groups."""
    hg, ho = res["gpu"]["hist"], res["orc"]["hist"]
    G = hg.shape[0]
    fg = hg / hg.sum(axis=1, keepdims=True)
    fo = ho / ho.sum(axis=1, keepdims=True)
    d = fg.mean(axis=0) - fo.mean(axis=0)
    var = fg.var(axis=0, ddof=1) / G + fo.var(axis=0, ddof=1) / G
    use = (hg.sum(axis=0) >= 20 * G) & (ho.sum(axis=0) >= 20 * G) & (var > 0)
    z = d[use] / np.sqrt(var[use])
    return float(np.sum(z * z)), int(use.sum()), float(np.max(np.abs(z)))


def _chi2_bound(nu, groups):
    """Acceptance bound for the chi-square of nu bins whose variances are estimated from
    `groups` samples per side: each term is close to a Student-t square with about
    2 (groups - 1) degrees of freedom (mean k / (k - 2), variance 2 k^2 (k - 1) / ((k - 2)^2
    (k - 4))); allow the mean plus five standard deviations of the sum."""
    k = 2 * (groups - 1)
    m = k / (k - 2)
    v = 2 * k * k * (k - 1) / ((k - 2) ** 2 * (k - 4))
    return nu * m + 5 * np.sqrt(nu * v)


def test_he3_ensemble_agrees_with_fp64_oracle():
    sysm = _he3()
    G, Wg = 16, 128
    ka = _he3_ka(sysm, walkers=Wg, op_runs=5, msteps=4)
    res = _ensemble(
        make_gpu=lambda gi: _gpu_kernel(sysm, ka, seed=100 + gi, fast=True),
        make_orc=lambda gi: _orc_fp64_ranlux(sysm, ka, gi),
        init_paths=lambda gi: sysm.initial_paths(Wg, 256, np.random.RandomState(500 + gi)),
        groups=G, burn_launches=1, launches=2, nops=1, hist=True)
    z = _z_operators(res, ["energy"])
    chi2, nu, zmax = _chi2_hist(res)
    print(f"\nHe3 T=1K: energy GPU {z['energy'][1]:.5f} K, oracle FP64 {z['energy'][2]:.5f} K, "
          f"se {z['energy'][3]:.5f}, z = {z['energy'][0]:.2f}; histogram chi2 = {chi2:.1f} over {nu} bins "
          f"(bound {_chi2_bound(nu, G):.1f}), max |z| = {zmax:.2f}")
    assert abs(z["energy"][0]) < 3.0
    assert nu > 40
    assert chi2 < _chi2_bound(nu, G)
    assert zmax < 5.0


def _orc_fp64_ranlux(sysm, ka, gi):
    o = _oracle(sysm, ka, double=True)
    o.init_ranlux_rows(o.ranlux_tab, (np.uint64(900 + gi) << np.uint64(32))
                       + np.arange(o.ranlux_tab.shape[0], dtype=np.uint64))
    o.init_ranlux_rows(o.group_tab, (np.uint64(950 + gi) << np.uint64(32))
                       + np.arange(o.group_tab.shape[0], dtype=np.uint64))
    o.walker_means = lambda: _oracle_walker_means(o, ka)
    return o


def test_bound_trimer_example_ensemble_agrees_with_fp64_oracle():
    """Lm2m2_3part at beta = 1000 (15 mK), the reference example's set-up at N = 16: bound,
    so the ensemble is stationary after burn-in."""
    from feynsimul_gb300.physical_systems.lm2m2_3part import Lm2m2_3part
    kernel, kernel_args = engine()
    sysm = Lm2m2_3part()
    G, Wg, N, S = 16, 64, 16, 2
    ops = (sysm.energyOp, sysm.meanSquaredRadiusOp, sysm.meanRadiusOp)
    ka = dict(nbrOfWalkers=Wg, N=N, beta=1000.0, S=S, enableOperator=True, enableCorrelator=False,
              enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
              nbrOfWalkersPerWorkGroup=4, enableParallelizePath=True, enableGlobalPath=True,
              enableGlobalOldPath=True, enableDouble=False, enableRanlux=False, luxuaryFactor=2,
              ranluxIntMax=2 ** 32 - 1, operators=ops, operatorRuns=25, metroStepsPerOperatorRun=40)

    def make_gpu(gi):
        return kernel.PIMCKernel(kernel_args.KernelArgs(system=sysm, seed=300 + gi, fastMath=True, **ka))

    def make_orc(gi):
        o = _oracle(sysm, ka, double=True, hist=False)
        rs = np.random.RandomState(700 + gi)
        o.seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.seeds.shape)
        o.walker_seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape)
        nT = o.op_means.size // len(ops)
        T = N // 2 ** S

        def walker_means():
            # work-item ids of 4 walkers per work group (kernel.c:539-541)
            per = o.op_means.reshape(nT, len(ops))
            WPG, nWG = 4, Wg // 4
            w = np.arange(Wg)
            tid = ((w // WPG) * T + (w % WPG) * nWG * T)[:, None] + np.arange(T)[None, :]
            return per[tid].mean(axis=1).T
        o.walker_means = walker_means
        return o

    def init_paths(gi):
        # the example's start: every slice at one point U(-1, 1) * 0.01 per coordinate
        start = np.random.RandomState(40 + gi).uniform(size=(Wg, sysm.DOF), low=-1.0, high=1.0) * 0.01
        return np.ascontiguousarray(np.repeat(start[:, :, None], N, axis=2).reshape(Wg, sysm.DOF * N))

    res = _ensemble(make_gpu, make_orc, init_paths, groups=G, burn_launches=2, launches=2, nops=3, hist=False)
    z = _z_operators(res, ["energy", "msr", "mean_radius"])
    print("\nLm2m2_3part beta=1000 N=16: " + "; ".join(
        f"{n} GPU {v[1]:.6g} oracle {v[2]:.6g} se {v[3]:.2g} z {v[0]:.2f}" for n, v in z.items()))
    for name, v in z.items():
        assert np.isfinite(v[0]) and abs(v[0]) < 3.0, (name, v)
