"""The sweeps' status word: a path value that is not finite after a launch is reported by
fs_sync as FS_ERR_NUMERIC, naming the walker, and the word is cleared once read.

The failure is made on the host: one walker's path is set to NaN (every slice, so no move
can replace it: a midpoint of NaN endpoints is NaN).  Nothing faults: the kernels only
read and write in-bounds values and compare them."""
import types

import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("global_path", [False, True], ids=["shared_path", "global_path"])
def test_nonfinite_path_is_reported_and_cleared(global_path):
    require_gpu()
    kernel, kernel_args = engine()
    from feynsimul_gb300 import _lib
    sysm = types.SimpleNamespace(DOF=2, potential="0.5 * (x1 * x1 + x2 * x2)", userCode="")
    W, N = 64, 32
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=W, N=N, beta=4.0, S=2, enableOperator=True, enableCorrelator=False,
        enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
        nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=global_path,
        enableGlobalOldPath=False, operators=("x1 * x1",), operatorRuns=2, metroStepsPerOperatorRun=2, seed=3)
    k = kernel.PIMCKernel(ka)
    clean = np.random.RandomState(1).randn(W, N * 2).astype(np.float32) * 0.5
    k.setPaths(clean)
    k.run()                                   # finite paths: no error
    bad = clean.copy()
    bad[37] = np.nan
    k.setPaths(bad)
    with pytest.raises(_lib.FsError) as e:
        k.run()
    assert e.value.code == _lib.FS_ERR_NUMERIC
    assert "walker 37" in str(e.value)
    assert np.isnan(k.getPaths()[37]).all()
    assert np.isfinite(np.delete(k.getPaths(), 37, axis=0)).all()
    k.setPaths(clean)
    k.run()                                   # the word was cleared: the next run is clean
    # the polling wait reports the same way
    k.setPaths(bad)
    k.run(wait=False)
    rc = _lib.lib().fs_sync_timeout(k._handle, 30.0)
    assert rc == _lib.FS_ERR_NUMERIC
    k.close()
