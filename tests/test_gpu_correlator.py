"""Correlator partial sums on the GPU: the default FP32 partials (four fused multiply-add
chains per lag and measurement) against float-float partials of the same trajectory.

Both add one FP64 term per lag and measurement to the running sums, and the moves do not
depend on the accumulation, so the paths are bit-identical and the running sums differ only
by the partials' rounding.  Bound per measurement, with u = 2^-24 and
gamma(n) = n u / (1 - n u): the FMA partial is within gamma(N/4 + 2) * sum_s |a_s a_(s+tau)|
of the exact sum, and the float-float sum of the rounded products within
(u + 2^-44) * sum_s |a_s a_(s+tau)|; by Cauchy-Schwarz sum_s |a_s a_(s+tau)| <= sum_s a_s^2,
the lag-0 term.  Summed over measurements: |fp32 - float-float| <= (gamma + 2u) * C(0).

Also: the pipelined correlator helpers (lag sums one measurement behind the moves) give the
same bits as helpers that wait for the moves."""
import types

import numpy as np
import pytest

from gpu_util import engine, require_gpu

pytestmark = pytest.mark.gpu


COR2 = ("x1", "x1 * x1 - 0.5")
# five correlators: more than the lag sums keep in registers (4 lags x 4 correlators)
COR5 = ("x1", "x1 * x1 - 0.5", "x1 * x1 * x1", "0.5 * x1 + 0.25", "x1 * x1 * x1 * x1 - 0.75")


def _kernel(partials, parallel, N, S, W=256, wpb=0, fast=True, cors=COR2, accumulation="fp64"):
    kernel, kernel_args = engine()
    sysm = types.SimpleNamespace(DOF=1, potential="0.5 * x1 * x1", userCode="")
    ka = kernel_args.KernelArgs(
        system=sysm, nbrOfWalkers=W, N=N, beta=10.0, S=S, enableOperator=True, enableCorrelator=True,
        enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
        nbrOfWalkersPerWorkGroup=1, enableParallelizePath=parallel, enableGlobalPath=False,
        enableGlobalOldPath=False, operators=("x1 * x1",), correlators=cors,
        operatorRuns=6, metroStepsPerOperatorRun=2, partials=partials, walkersPerBlock=wpb,
        fastMath=fast, accumulation=accumulation, seed=11)
    return kernel.PIMCKernel(ka)


@pytest.mark.parametrize("parallel,N,S,wpb", [
    (True, 128, 3, 0),   # 16 segment threads + 16 pipelined helpers, 4 lags each
    (True, 64, 2, 0),    # 16 segment threads + 16 pipelined helpers, 8 of them 4 lags each
    (True, 128, 3, 1),   # movers in half warps: 16 + 48 helpers after the moves, one lag each
    (True, 256, 2, 0),   # 64 segment threads, two lags each, no helpers
    (False, 64, 2, 0),   # one thread per walker: all 32 lags in one loop, sums in device memory
], ids=["pipelined", "pipelined_n64", "helpers", "two_lags", "walker_mode"])
def test_fp32_partials_within_bound_of_float_float(parallel, N, S, wpb):
    require_gpu()
    W = 256
    kf, kx = _kernel("fp32", parallel, N, S, W, wpb), _kernel("exact", parallel, N, S, W, wpb)
    p0 = (np.random.RandomState(5).randn(W, N) * 0.7).astype(np.float32)
    for k in (kf, kx):
        k.setPaths(p0)
    for _ in range(3):
        kf.run()
        kx.run()
    assert np.array_equal(kf.getPaths(), kx.getPaths())
    a = kf._raw_correlator().reshape(W, 2, N // 2)
    b = kx._raw_correlator().reshape(W, 2, N // 2)
    u = 2.0 ** -24
    n = N // 4 + 2
    bound = (n * u / (1 - n * u) + 2 * u) * b[:, :, :1]
    err = np.abs(a - b)
    assert np.all(err <= bound), (err / bound).max()
    assert np.all(b[:, :, 0] > 0)
    # the bound resolves the values: far below the statistical spread of the lag sums
    assert bound.max() < 1e-4 * b[:, :, 0].std()
    kf.close()
    kx.close()


@pytest.mark.parametrize("cors,accumulation", [(COR2, "fp64"), (COR5, "fp64"), (COR2, "kahan")],
                         ids=["two_correlators", "five_correlators", "kahan"])
def test_pipelined_helpers_bit_identical(cors, accumulation):
    """The launch shapes of one HO run (N = 128, S = 3: 16 segment threads per walker):
    2 walkers per CTA pipeline 16 helper threads per walker (4 lags each, the correlator
    values from a path snapshot) one measurement behind the movers; 1 walker per CTA leaves
    the movers in half warps, so every thread of 4 groups sums one lag after the moves.  Each sum is formed in the same order either way, so paths, operators, accepts
    and correlator sums are bit-identical.  IEEE builds:
    with contraction allowed, the compiler may fuse x1 * x1 - 0.5 into one FMA at one call
    site and not at another, and the two shapes evaluate it at different call sites."""
    require_gpu()
    W, N = 256, 128
    kp = _kernel("fp32", True, N, 3, W, wpb=2, fast=False, cors=cors, accumulation=accumulation)
    kh = _kernel("fp32", True, N, 3, W, wpb=1, fast=False, cors=cors, accumulation=accumulation)
    assert (kp._info.walkers_per_block, kp._info.block_threads) == (2, 2 * 16 * 2)
    assert (kh._info.walkers_per_block, kh._info.block_threads) == (1, 16 * 4)
    p0 = (np.random.RandomState(6).randn(W, N) * 0.7).astype(np.float32)
    for k in (kp, kh):
        k.setPaths(p0)
    for _ in range(3):
        kp.run()
        kh.run()
    assert np.array_equal(kp.getPaths(), kh.getPaths())
    assert np.array_equal(kp._raw_operators(), kh._raw_operators())
    assert np.array_equal(kp.getAccepts(), kh.getAccepts())
    assert np.array_equal(kp._raw_correlator(), kh._raw_correlator())
    kp.close()
    kh.close()


@pytest.mark.parametrize("N,S", [(32, 2), (64, 3), (64, 2), (128, 4), (256, 4)])
def test_pipelined_helpers_bit_identical_across_shapes(N, S):
    """Pipelined helpers (walkers per CTA filling whole warps of movers) against the same run
    with one walker per CTA (helpers after the moves, or none): identical bits, IEEE build."""
    require_gpu()
    W, tpw = 64, N >> S
    kp = _kernel("fp32", True, N, S, W, wpb=32 // tpw, fast=False)
    kh = _kernel("fp32", True, N, S, W, wpb=1, fast=False)
    groups = -(-(N // 8) // tpw)
    assert kp._info.block_threads == (32 // tpw) * tpw * (1 + groups)
    p0 = (np.random.RandomState(N + S).randn(W, N) * 0.7).astype(np.float32)
    for k in (kp, kh):
        k.setPaths(p0)
    for _ in range(2):
        kp.run()
        kh.run()
    assert np.array_equal(kp.getPaths(), kh.getPaths())
    assert np.array_equal(kp._raw_operators(), kh._raw_operators())
    assert np.array_equal(kp._raw_correlator(), kh._raw_correlator())
    kp.close()
    kh.close()
