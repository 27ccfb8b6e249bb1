"""GPU parity: the CUDA engine (through the C ABI) against the reference's own kernel.c run
on the CPU (golden fixtures) and against the oracle restatement.

Tolerances: integer results (seed tables, RANLUX states, generator streams) must be
bit-exact.  Floating-point results use the same IEEE operations in the same order; only
CUDA's and the C library's log / sin / exp may round differently in the last ulp, so
paths and sums are compared with rtol 1e-4, and an accept decision may flip where
exp(dS) lies within ~1e-6 of its uniform (at most one flip is tolerated per case).
"""
import numpy as np
import pytest

from golden_cases import load_ranlux, load_sweep, oracle_config, sweep_cases
from gpu_util import kernel_for_case, masked, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


# ---------------------------------------------------------------- generator streams
@pytest.mark.parametrize("lux", [0, 1, 2, 3, 4, 124])
def test_ranlux_stream_bit_exact(lux):
    from feynsimul_gb300 import _lib
    L = _lib.lib()
    g = load_ranlux()
    xs = np.ascontiguousarray(g["seeds"].astype(np.uint64))
    n = xs.shape[0]
    out = np.zeros((n, 400), np.float32)
    st = np.zeros((n, 28), np.uint32)
    _lib.check(L.fs_rng_ranlux_stream(lux, xs.ctypes.data, n, 100, out.ctypes.data, st.ctypes.data))
    assert np.array_equal(out.view(np.uint32), g[f"f32_lux{lux}"].view(np.uint32))
    assert np.array_equal(masked(st), g[f"state_lux{lux}"])
    out64 = np.zeros((2, 160), np.float64)
    _lib.check(L.fs_rng_ranlux_stream64(lux, xs[:2].copy().ctypes.data, 2, 40, out64.ctypes.data))
    assert np.array_equal(out64, g[f"f64_lux{lux}"])


def test_xorshift_stream_bit_exact():
    from feynsimul_gb300 import _lib
    from oracle import oracle as orc
    L = _lib.lib()
    rng = np.random.RandomState(4)
    st = rng.randint(0, 2 ** 31 - 1, size=(64, 4)).astype(np.uint32)
    ints = np.zeros((64, 500), np.uint32)
    flts = np.zeros((64, 500), np.float32)
    st_gpu = st.copy()
    _lib.check(L.fs_rng_xorshift_stream(st_gpu.ctypes.data, 64, 500, ints.ctypes.data, flts.ctypes.data))
    for i in range(64):
        ref, fin = orc.xorshift_stream(st[i], 500)
        assert np.array_equal(ints[i], ref)
        assert np.array_equal(st_gpu[i], fin)
        # kernel.c:229 under single-precision constants: float(w) * 2^-32
        assert np.array_equal(flts[i], ref.astype(np.float32) * np.float32(2.0 ** -32))


# ---------------------------------------------------------------- sweeps vs reference
@pytest.mark.parametrize("global_path", [True, False], ids=["global_path", "shared_path"])
@pytest.mark.parametrize("case", sweep_cases())
def test_sweep_matches_reference_kernel(case, global_path):
    ka, rec = load_sweep(case)
    ka = dict(ka, enableGlobalPath=global_path)
    k = kernel_for_case(ka, compat=True, accumulation="fp32", fast=False)
    k.setPaths(rec["paths0"])
    if ka["enableRanlux"]:
        k.setRanluxTables(rec["ranlux_tab0"], rec["group_tab0"])
    else:
        k.setSeeds(rec["seeds0"])
    flips_total = 0
    for it in (1, 2):
        k.run()
        if ka["enableRanlux"]:
            t, g = k.getRanluxTables()
            assert np.array_equal(masked(t), rec[f"ranlux_tab{it}"])
            assert np.array_equal(masked(g), rec[f"group_tab{it}"])
        else:
            assert np.array_equal(k.getSeeds(), rec[f"seeds{it}"])
        acc = k.getAccepts()
        flips_total += int((acc != rec[f"accepts{it}"]).sum())
        assert flips_total <= 1, (acc, rec[f"accepts{it}"])
        if flips_total == 0:
            np.testing.assert_allclose(k.getPaths(), rec[f"paths{it}"], rtol=1e-4, atol=1e-5)
            raw = k._raw_operators()
            np.testing.assert_allclose(raw, rec[f"ops{it}"], rtol=1e-4, atol=1e-5)
            cor = k._raw_correlator()
            np.testing.assert_allclose(cor.reshape(rec[f"cor{it}"].shape), rec[f"cor{it}"], rtol=1e-4, atol=1e-4)
            assert np.abs(k.getBinCountsRaw().astype(np.int64) - rec[f"bins{it}"].astype(np.int64)).sum() <= 2
    k.close()


# ---------------------------------------------------------------- fixed mode vs oracle
FIXED_CASES = {
    "xorshift_parallel": {},
    "xorshift_walker": {},
    "ranlux_parallel_lux2": dict(nbrOfWalkers=8, nbrOfWalkersPerWorkGroup=2),
    "ranlux_walker_lux0": {},
    "xorshift_parallel_double": {},
    "xorshift_walker_moves": {},
    "xorshift_walker_snm_only": {},
    "ranlux_walker_moves": {},
    "xorshift_walker_shift_double": {},
    # edge geometries of the correlator sums: one lag per thread; one thread per walker
    # owning 4 lags; walker mode whose 4 lags take the one-pass loop
    "xorshift_parallel:n4_s1": dict(N=4, S=1),
    "xorshift_parallel:n8_s3": dict(N=8, S=3),
    "xorshift_walker:n8": dict(N=8),
    # a walker count no CTA shape divides (the last CTA holds inactive walkers), and walkers
    # of more than 32 segment threads (one walker per CTA, block-wide barriers)
    "xorshift_parallel:w13": dict(nbrOfWalkers=13, nbrOfWalkersPerWorkGroup=1),
    "xorshift_parallel:n512_s2": dict(N=512, S=2, nbrOfWalkers=4, nbrOfWalkersPerWorkGroup=1),
    # the largest walker: 1024 segment threads, 4096 correlator lags of 8192 products
    "xorshift_parallel:n8192_s3": dict(N=8192, S=3, nbrOfWalkers=2, nbrOfWalkersPerWorkGroup=1),
}


def _oracle_correlator(o, accum):
    """The oracle's correlator sums in the layout fs_get_correlator returns."""
    if accum == 3:
        c = o.cor_means
        return np.stack([c["f"], c["ks"], c["kc"], c["d"]], axis=-1).astype(np.float64).reshape(-1)
    return o.cor_means.astype(np.float64).reshape(-1)


@pytest.mark.parametrize("global_path", [False, True], ids=["shared_path", "global_path"])
@pytest.mark.parametrize("case", sorted(FIXED_CASES))
@pytest.mark.parametrize("accum", [1, 0, 2, 3])
def test_fixed_mode_matches_oracle(case, accum, global_path):
    from oracle import oracle as orc
    ka, rec = load_sweep(case.split(":")[0])
    ka = dict(ka, enableGlobalPath=global_path, **FIXED_CASES[case])
    accname = {0: "fp32", 1: "fp64", 2: "kahan", 3: "study"}[accum]
    k = kernel_for_case(ka, compat=False, accumulation=accname, fast=False)
    o = orc.OracleSampler(oracle_config(ka, compat=False, accum=accum))
    rng = np.random.RandomState(21)
    p0 = (rng.randn(*o.paths.shape) * 0.4).astype(o.paths.dtype)
    o.paths[...] = p0
    k.setPaths(p0)
    if ka["enableRanlux"]:
        k.initRanlux()
        k.groupInitRanlux()
        t, g = k.getRanluxTables()
        o.ranlux_tab[...] = t
        o.group_tab[...] = g
        # the GPU's table seeding equals the oracle's ranluxcl_init
        o2 = orc.OracleSampler(oracle_config(ka, compat=False, accum=accum))
        o2.init_ranlux_rows(o2.ranlux_tab, (np.uint64(int(k._seeds[0])) << np.uint64(32))
                            + np.arange(o2.ranlux_tab.shape[0], dtype=np.uint64))
        assert np.array_equal(o2.ranlux_tab, t)
    else:
        o.seeds[...] = k.getSeeds()
        o.walker_seeds[...] = k.getWalkerSeeds()
    flips = 0
    for it in range(2):
        k.run()
        o.run()
        if ka["enableRanlux"]:
            t, g = k.getRanluxTables()
            assert np.array_equal(t, o.ranlux_tab)
            assert np.array_equal(g, o.group_tab)
        else:
            assert np.array_equal(k.getSeeds(), o.seeds)
            assert np.array_equal(k.getWalkerSeeds(), o.walker_seeds)
        flips += int((k.getAccepts() != o.accepts).sum())
        assert flips <= 1
        if flips == 0:
            np.testing.assert_allclose(k.getPaths(), o.paths, rtol=1e-4, atol=1e-5)
            raw = k._raw_operators()
            np.testing.assert_allclose(raw, o.op_means.reshape(-1)[:raw.size], rtol=1e-4, atol=1e-5)
            if ka["enableCorrelator"]:
                cor = k._raw_correlator()
                want = _oracle_correlator(o, accum)
                assert cor.size == want.size
                np.testing.assert_allclose(cor, want, rtol=1e-4, atol=1e-4)
            assert np.array_equal(k.getBinCountsRaw(), o.bins) or \
                np.abs(k.getBinCountsRaw().astype(np.int64) - o.bins.astype(np.int64)).sum() <= 2
    k.close()
