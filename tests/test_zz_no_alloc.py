"""fs_ranlux_init_noalloc: seeding a RANLUX table with no device allocation by the library.

For callers that cannot let a library call cudaMalloc (their memory pool owns the device
memory, or their binding's allocator must own every buffer): the entry point stages the
seed values in a fixed scratch array inside the library and writes the caller's own table.
This file is collected last so that a run stopping at its first failure has already run
every other test.  Each call here goes through the C ABI and is compared with the
existing entry point, fs_ranlux_init on a handle, which must agree bit for bit (the
seeding is integer work)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference_tables(xs):
    """Seed the same rows through the existing entry point (a walker-mode handle has one
    table row per walker)."""
    import types
    from feynsimul_gb300.kernel import PIMCKernel
    from feynsimul_gb300.kernel_args import KernelArgs
    n = xs.shape[0]
    sysm = types.SimpleNamespace(DOF=1, potential="x1*x1", userCode="")
    ka = KernelArgs(system=sysm, nbrOfWalkers=n, N=8, beta=1.0, S=1, enableOperator=False,
                    enableCorrelator=False, enableBisection=True, enablePathShift=False,
                    enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
                    enableParallelizePath=False, enableGlobalPath=False, enableGlobalOldPath=False,
                    enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1, operatorRuns=1,
                    metroStepsPerOperatorRun=1)
    k = PIMCKernel(ka)
    from feynsimul_gb300 import _lib
    _lib.check(_lib.lib().fs_ranlux_init(k._handle, xs.ctypes.data, n), k._handle)
    tab, _ = k.getRanluxTables()
    k.close()
    return tab


def test_noalloc_matches_existing_entry_point_twice():
    from gpu_util import require_gpu
    require_gpu()
    import torch
    from feynsimul_gb300 import _lib
    from feynsimul_gb300 import build
    build.build()
    L = _lib.lib()
    rng = np.random.RandomState(2024)
    for n in (3000, 1777):  # two calls in a row, the second shorter than the first
        xs = np.ascontiguousarray(rng.randint(0, 2 ** 62, size=n, dtype=np.int64).astype(np.uint64))
        table = torch.zeros(n * 28, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(L.fs_ranlux_init_noalloc(ctypes.c_void_p(table.data_ptr()), xs.ctypes.data, n,
                                            ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        got = table.cpu().numpy().view(np.uint32).reshape(n, 28)
        want = _reference_tables(xs)
        assert np.array_equal(got, want)


def test_noalloc_rejects_too_many_rows():
    from gpu_util import require_gpu
    require_gpu()
    from feynsimul_gb300 import _lib
    L = _lib.lib()
    n = (1 << 18) + 1
    xs = np.zeros(n, np.uint64)
    rc = L.fs_ranlux_init_noalloc(ctypes.c_void_p(16), xs.ctypes.data, n, None)
    assert rc == _lib.FS_ERR_CONFIG
    assert b"262144" in L.fs_last_error(None)
