"""The potential cache (V of every slice kept between moves, so the old action is a sum of
cached values and a move evaluates the potential only at its proposed nodes) in shared memory
(potentialCache=True) and in device memory (potentialCache="device") against the sweep without
it (potentialCache=False): the old action is the same products and sums of the same values,
so paths, accept counts, operator sums and RANLUX tables are bit-identical (IEEE builds:
with contraction allowed the compiler may fuse the potential's arithmetic differently at
different call sites)."""
import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


def _he3_kernel(pc, walkers=64, global_path=False, parallel=True, S=4, N=256):
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    kernel, kernel_args = engine()
    sysm = Lm2m2Cluster(3, 1.0)
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=walkers, N=N, beta=float(sysm.beta), S=S, enableOperator=True,
        enableCorrelator=False, enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
        enableBins=False, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=parallel,
        enableGlobalPath=global_path, enableGlobalOldPath=False, enableDouble=False, enableRanlux=True,
        luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1, operators=(sysm.energyOp,), operatorRuns=2,
        metroStepsPerOperatorRun=3, fastMath=False, potentialCache=pc, seed=17,
        histograms=sysm.pairDistanceOps, histRange=(0.0, 20.0), histBins=200)
    k = kernel.PIMCKernel(ka)
    k.initRanlux()
    k.groupInitRanlux()
    return k, sysm


def _same_run(kernels, p0, launches=2):
    for k in kernels:
        k.setPaths(p0)
    for _ in range(launches):
        for k in kernels:
            k.run()
    ref = kernels[0]
    for k in kernels[1:]:
        assert np.array_equal(k.getPaths(), ref.getPaths())
        assert np.array_equal(k.getAccepts(), ref.getAccepts())
        assert np.array_equal(k._raw_operators(), ref._raw_operators())
        t, g = k.getRanluxTables()
        t0, g0 = ref.getRanluxTables()
        assert np.array_equal(t, t0) and np.array_equal(g, g0)
        assert np.array_equal(k.getHistogram(density=False)[1], ref.getHistogram(density=False)[1])
    assert ref.getAccepts().sum() > 0


@pytest.mark.parametrize("global_path,parallel,S", [(False, True, 4), (True, True, 4), (False, True, 2),
                                                     (False, False, 3)],
                         ids=["shared_path", "global_path", "s2", "walker_mode"])
def test_potential_cache_bit_identical(global_path, parallel, S):
    require_gpu()
    W = 64
    ks = [_he3_kernel(pc, W, global_path, parallel, S)[0] for pc in (False, True, "device")]
    sysm = _he3_kernel(False, 1)[1]
    p0 = sysm.initial_paths(W, 256, np.random.RandomState(23)).astype(np.float32)
    _same_run(ks, p0)
    # the device-memory cache costs no shared memory
    assert ks[2]._info.smem_bytes == ks[0]._info.smem_bytes
    for k in ks:
        k.close()


def test_potential_cache_automatic_choice():
    """The bench's He3 shape (4 walkers per CTA, shared memory full with their paths) takes
    the cache in device memory; a 1-DOF oscillator takes none there (its potential costs
    less than a cache load and store)."""
    require_gpu()
    import types
    kernel, kernel_args = engine()
    k = _he3_kernel(None, 256)[0]
    assert k._info.potential_cache == 3
    k.close()
    sysm = types.SimpleNamespace(DOF=1, potential="0.5 * x1 * x1", userCode="")
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=256, N=128, beta=10.0, S=3, enableOperator=True, enableCorrelator=False,
        enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
        nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
        enableGlobalOldPath=False, operators=("x1 * x1",), operatorRuns=2, metroStepsPerOperatorRun=2,
        seed=3)
    k = kernel.PIMCKernel(ka)
    assert k._info.potential_cache in (0, 1)
    k.close()


def test_potential_cache_device_chunked_host_run():
    """fs_run_host's chunked launches (each chunk a block offset into the walkers) with the
    device-memory cache: the same result as set / run / get without the cache."""
    require_gpu()
    W = 4096
    ka_, kb_ = _he3_kernel(False, W)[0], _he3_kernel("device", W)[0]
    sysm = _he3_kernel(False, 1)[1]
    p0 = sysm.initial_paths(W, 256, np.random.RandomState(29)).astype(np.float32)
    ka_.setPaths(p0)
    ka_.run()
    out = np.empty_like(p0)
    kb_.runHost(p0, out=out, chunks=3)
    assert np.array_equal(out.reshape(-1), ka_.getPaths().reshape(-1))
    assert np.array_equal(kb_.getAccepts(), ka_.getAccepts())
    ka_.close()
    kb_.close()
