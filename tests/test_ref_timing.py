"""The reference-timing launcher (oracle/ref_timing.py; CPU only): the reference's own kernel
run with the work-items of each work-group as fibers, its __local path array shared by the
group, gives bit for bit what oracle/build_ref.py's one-thread-per-work-item launcher gives
on the global-path build of the same configuration (IEEE flags on both).  Needs the
reference tree (where bench.py's reference arm is prepared)."""
import numpy as np
import pytest

from oracle import build_ref

pytestmark = pytest.mark.skipif(not build_ref.reference_available(), reason="reference tree absent")


def _he3_ka(global_path, walkers=4):
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    sysm = Lm2m2Cluster(3, 1.0)
    ka = dict(nbrOfWalkers=walkers, N=64, beta=float(sysm.beta), S=3, enableOperator=True,
              enableCorrelator=False, enableBisection=True, enablePathShift=False,
              enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
              enableParallelizePath=True, enableGlobalPath=global_path, enableGlobalOldPath=False,
              enableDouble=False, enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
              operators=(sysm.energyOp,), operatorRuns=2, metroStepsPerOperatorRun=3)
    return sysm, ka


def test_fiber_work_groups_match_thread_per_work_item():
    from oracle import ref_timing
    sysm, ka_local = _he3_ka(False)
    _, ka_global = _he3_ka(True)
    ref_timing.prepare("test_he3", sysm, ka_local)
    fk = ref_timing.FiberKernel("test_he3", fast=False)
    rk = build_ref.RefKernel(ka_global, sysm, np_seed=0)
    p0 = sysm.initial_paths(4, 64, np.random.RandomState(5)).astype(np.float32)
    fk.init_ranlux(2)
    rk.init_ranlux()
    rk.group_init_ranlux()
    # word 25 of a 28-word RANLUXCL state is padding that ranluxcl_init leaves as it finds it
    live = np.arange(28) != 25
    for a, b in ((fk.bufs[-2], rk.k._ranluxcltab.arr), (fk.bufs[-1], rk.k._groupRanluxcltab.arr)):
        assert np.array_equal(a.reshape(-1, 28)[:, live], b.reshape(-1, 28)[:, live])
    fk.set_paths(p0)
    rk.set_paths(p0)
    for _ in range(2):
        fk.run(2)
        rk.run()
    assert np.array_equal(fk.bufs[0], rk.k._paths.arr)          # paths
    assert np.array_equal(fk.bufs[1], rk.k._accepts.arr)        # accept counts
    assert np.array_equal(fk.bufs[2], rk.k._operatorValues.arr)  # operator sums
    assert rk.k._accepts.arr.sum() > 0


def test_fiber_work_groups_with_the_correlators_barriers():
    """The harmonic oscillator with its correlator: a work-group barrier per lag and slice
    (kernel.c:792), 2 walkers in one work group; fibers against one thread per work-item.
    One work-group: in this xorshift mode every work-item reads the shared offset-seed row at
    its start and writes it at its end (kernel.c:568-572, :832-835), so work-groups that run
    one after another see each other's writes and the launch order would matter."""
    import types
    from oracle import ref_timing
    sysm = types.SimpleNamespace(DOF=1, potential="0.5*x1*x1", userCode="")

    def ka(global_path):
        return dict(nbrOfWalkers=2, N=16, beta=4.0, S=2, enableOperator=True, enableCorrelator=True,
                    enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
                    nbrOfWalkersPerWorkGroup=2, enableParallelizePath=True, enableGlobalPath=global_path,
                    enableGlobalOldPath=False, enableDouble=False, enableRanlux=False,
                    operators=("x1*x1",), correlators=("x1",), operatorRuns=3, metroStepsPerOperatorRun=2)
    ref_timing.prepare("test_ho", sysm, ka(False))
    fk = ref_timing.FiberKernel("test_ho", fast=False)
    rk = build_ref.RefKernel(ka(True), sysm, np_seed=0)
    p0 = (np.random.RandomState(8).randn(2, 16) * 0.5).astype(np.float32)
    fk.set_paths(p0)
    rk.set_paths(p0)
    fk.run(2)
    rk.run()
    for i, b in enumerate(rk.bufs):   # paths, accepts, seed rows, operator and correlator sums
        assert np.array_equal(fk.bufs[i], b.arr), i
    assert rk.k._accepts.arr.sum() > 0


def test_rate_of_a_prepared_sample():
    from oracle import ref_timing
    sysm, ka = _he3_ka(False, walkers=8)
    ref_timing.prepare("test_he3_rate", sysm, ka)
    assert ref_timing.available("test_he3_rate") and ref_timing.matches("test_he3_rate", ka)
    assert not ref_timing.matches("test_he3_rate", dict(ka, S=2))
    p0 = sysm.initial_paths(8, 64, np.random.RandomState(6)).astype(np.float32)
    r = ref_timing.rate("test_he3_rate", p0, seconds=0.2, threads=2)
    assert r["value"] > 0 and r["launches"] >= 1
    assert r["node_updates"] == r["launches"] * 8 * 8 * 7 * 6
