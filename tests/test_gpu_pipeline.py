"""The pipelined host-buffer run (fs_run_host / PIMCKernel.runHost) against
setPaths + run + getPaths: bit-identical paths, seed tables, accepts and sums, for several
chunk counts, both generators, and the walker-mode moves."""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()
    engine()


def _pair(ranlux, walker_mode=False, compat=False):
    kernel, kernel_args = engine()
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    sysm = Lm2m2Cluster(3, 1.0)
    ks = []
    for _ in range(2):
        ka = kernel_args.KernelArgs(
            system=sysm, nbrOfWalkers=200 if not walker_mode else 96, N=64, beta=sysm.beta, S=3,
            enableOperator=True, enableCorrelator=True, enableBisection=True,
            enablePathShift=walker_mode, PSAlpha=0.3, enableSingleNodeMove=walker_mode, alpha=0.4,
            enableBins=False, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=not walker_mode,
            enableGlobalPath=False, enableGlobalOldPath=False, enableRanlux=ranlux, luxuaryFactor=1,
            ranluxIntMax=2 ** 32 - 1, operators=(sysm.energyOp,), correlators=("x1",), operatorRuns=2,
            metroStepsPerOperatorRun=3, compat=compat, seed=4,
            histograms=sysm.pairDistanceOps, histRange=(0.0, 20.0), histBins=50)
        k = kernel.PIMCKernel(ka)
        if ranlux:
            k.initRanlux()
            k.groupInitRanlux()
        ks.append(k)
    p0 = sysm.initial_paths(ks[0]._nbrOfWalkers, 64, np.random.RandomState(3)).astype(np.float32)
    return ks, p0


@pytest.mark.parametrize("chunks", [0, 1, 3, 4, 64])
@pytest.mark.parametrize("ranlux,compat", [(False, False), (True, False), (False, True)],
                         ids=["xorshift", "ranlux", "xorshift_compat"])
def test_run_host_equals_set_run_get(ranlux, compat, chunks):
    (a, b), p0 = _pair(ranlux, compat=compat)
    a.setPaths(p0)
    for _ in range(2):
        a.run(launches=2)
    pa = a.getPaths()
    host = p0.copy()
    b.pinHost(host)
    try:
        for _ in range(2):
            b.runHost(host, out=host, launches=2, chunks=chunks)
    finally:
        b.unpinHost(host)
    assert np.array_equal(pa, host)
    assert np.array_equal(a.getAccepts(), b.getAccepts())
    assert np.array_equal(a._raw_operators(), b._raw_operators())
    assert np.array_equal(a._raw_correlator(), b._raw_correlator())
    assert np.array_equal(a.getHistogram(density=False)[1], b.getHistogram(density=False)[1])
    if ranlux:
        ta, ga = a.getRanluxTables()
        tb, gb = b.getRanluxTables()
        assert np.array_equal(ta, tb) and np.array_equal(ga, gb)
    else:
        assert np.array_equal(a.getSeeds(), b.getSeeds())
    a.close()
    b.close()


@pytest.mark.parametrize("compat", [False, True])
def test_run_host_walker_moves(compat):
    (a, b), p0 = _pair(False, walker_mode=True, compat=compat)
    a.setPaths(p0)
    a.run(launches=3)
    host = p0.copy()
    out = b.runHost(host, launches=3, chunks=4)
    assert np.array_equal(a.getPaths(), out)
    assert np.array_equal(a.getAccepts(), b.getAccepts())
    a.close()
    b.close()
