"""The CPU oracle restatement against the golden fixtures made from the reference's
own kernel.c / RANLUXCL (tests/golden/make_golden.py), and, where the reference tree is
present, against the reference built live (oracle/build_ref.py)."""
import numpy as np
import pytest

from golden_cases import HO, load_ranlux, load_sweep, oracle_config, sweep_cases
from oracle import oracle as orc


@pytest.mark.parametrize("lux", [0, 1, 2, 3, 4, 124])
def test_ranlux_streams_bit_exact(lux):
    g = load_ranlux()
    for i, s in enumerate(g["seeds"]):
        out, st = orc.ranlux_stream(int(s), lux, 100)
        assert np.array_equal(out.view(np.uint32), g[f"f32_lux{lux}"][i].view(np.uint32))
        st = st.copy()
        st[25] = 0
        assert np.array_equal(st, g[f"state_lux{lux}"][i])
    for i, s in enumerate(g["seeds"][:2]):
        out, _ = orc.ranlux_stream(int(s), lux, 40, double=True)
        assert np.array_equal(out, g[f"f64_lux{lux}"][i])


@pytest.mark.parametrize("lux", [0, 2, 4])
def test_rng_moments_known_answer(lux):
    """The reference's examples/ranlux_test.py check: uniforms with mean 1/2 and standard
    deviation 1/sqrt(12), here on 10^6 values of the generators the golden streams pin
    (RANLUX per luxury level, xorshift as float(w) * 2^-32), at 6 standard errors."""
    out, _ = orc.ranlux_stream(123456789, lux, 250000)
    xs, _ = orc.xorshift_stream([123456789, 362436069, 521288629, 88675123], 1000000)
    for u in (out.astype(np.float64), xs.astype(np.float64) * 2.0 ** -32):
        n = u.size
        assert np.all((u >= 0.0) & (u < 1.0))
        assert abs(u.mean() - 0.5) < 6 * np.sqrt(1 / 12 / n)
        assert abs(u.std() - 1 / np.sqrt(12)) < 6 * np.sqrt(1 / 60 / n)     # Var(s) = (mu4 - s^4) / (4 s^2 n)


def _masked(t):
    t = np.array(t).reshape(-1, 28).copy()
    t[:, 25] = 0
    return t


@pytest.mark.parametrize("case", sweep_cases())
def test_sweep_matches_reference_golden(case):
    ka, rec = load_sweep(case)
    o = orc.OracleSampler(oracle_config(ka, compat=True, accum=0))
    o.paths[...] = rec["paths0"]
    if ka["enableRanlux"]:
        o.ranlux_tab[...] = rec["ranlux_tab0"]
        o.group_tab[...] = rec["group_tab0"]
    else:
        o.seeds[...] = rec["seeds0"]
    for it in (1, 2):
        o.run()
        # seed tables and accept counts: integer, bit-exact
        if ka["enableRanlux"]:
            assert np.array_equal(_masked(o.ranlux_tab), rec[f"ranlux_tab{it}"])
            assert np.array_equal(_masked(o.group_tab), rec[f"group_tab{it}"])
        else:
            assert np.array_equal(o.seeds, rec[f"seeds{it}"])
        assert np.array_equal(o.accepts, rec[f"accepts{it}"])
        assert np.array_equal(o.bins, rec[f"bins{it}"])
        # floats: same operations in the same order on IEEE hardware.  libm's
        # log/sin/exp may differ by an ulp between CPU families, hence the tolerance.
        np.testing.assert_allclose(o.paths, rec[f"paths{it}"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(o.op_means[:rec[f"ops{it}"].size], rec[f"ops{it}"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(o.cor_means, rec[f"cor{it}"], rtol=1e-5, atol=1e-5)


def test_ranlux_compat_quirks_visible_in_golden():
    """The reference seeds every per-thread RANLUX state from seeds[0] (kernel.c:155) and
    its RANLUX integers have zero low bits (kernel.c:206), so the bisection grid never
    shifts: slices 0, 4, 8, 12 keep their initial values."""
    ka, rec = load_sweep("ranlux_parallel_lux2")
    t0 = rec["ranlux_tab0"]
    assert (t0 == t0[0]).all()
    seg = 2 ** ka["S"]
    p0 = rec["paths0"].reshape(ka["nbrOfWalkers"], ka["N"])
    p2 = rec["paths2"].reshape(ka["nbrOfWalkers"], ka["N"])
    assert np.array_equal(p0[:, ::seg], p2[:, ::seg])
    assert not np.array_equal(p0, p2)


def test_oracle_against_live_reference():
    """Where the reference tree exists, rebuild it and compare once more (not a golden)."""
    from oracle import build_ref as br
    if not br.reference_available():
        pytest.skip("reference tree not present")
    import types
    from golden_cases import HO
    ka, _ = load_sweep("xorshift_parallel")
    r = br.RefKernel(dict(ka, nbrOfWalkers=4, N=32, S=3), types.SimpleNamespace(**HO), np_seed=3)
    o = orc.OracleSampler(oracle_config(dict(ka, nbrOfWalkers=4, N=32, S=3)))
    rng = np.random.RandomState(9)
    p0 = (rng.randn(*r.k._paths.arr.shape) * 0.5).astype(np.float32)
    r.k._paths.arr[...] = p0
    o.paths[...] = p0
    o.seeds[...] = r.k._seeds.arr
    r.run()
    o.run()
    assert np.array_equal(o.seeds, r.k._seeds.arr)
    assert np.array_equal(o.accepts, r.k._accepts.arr)
    assert np.array_equal(o.paths, r.k._paths.arr)


def test_oracle_against_live_reference_he3_bench_configuration():
    """The benchmarked configuration's arithmetic against the reference's own kernel: the He3
    trimer plugin, RANLUX luxuaryFactor 2, parallel-path mode with the path in __local
    memory (the reference kernel run with its work-groups as fibers, oracle/ref_timing.py,
    IEEE flags), N = 256, S = 4, 4 walkers, 2 launches; the oracle in the reference's
    compatible mode on the same RANLUX tables: tables, accept counts, paths and operator sums
    bit-exact (both sides call the same C library)."""
    from oracle import build_ref as br
    if not br.reference_available():
        pytest.skip("reference tree not present")
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    from oracle import ref_timing
    from oracle.oracle import OracleConfig, OracleSampler
    sysm = Lm2m2Cluster(3, 1.0)
    ka = dict(nbrOfWalkers=4, N=256, beta=float(sysm.beta), S=4, enableOperator=True,
              enableCorrelator=False, enableBisection=True, enablePathShift=False,
              enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
              enableParallelizePath=True, enableGlobalPath=False, enableGlobalOldPath=False,
              enableDouble=False, enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
              operators=(sysm.energyOp,), operatorRuns=2, metroStepsPerOperatorRun=3)
    ref_timing.prepare("test_he3_bench", sysm, ka)
    fk = ref_timing.FiberKernel("test_he3_bench", fast=False)
    o = OracleSampler(OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=4, N=256,
        beta=ka["beta"], S=4, operatorRuns=2, metroStepsPerOperatorRun=3, nbrOfWalkersPerWorkGroup=1,
        enableParallelizePath=True, enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
        operators=(sysm.energyOp,), compat=True, accum=0))
    fk.init_ranlux(2)
    o.ranlux_tab[...] = fk.bufs[-2].reshape(o.ranlux_tab.shape)
    o.group_tab[...] = fk.bufs[-1].reshape(o.group_tab.shape)
    p0 = sysm.initial_paths(4, 256, np.random.RandomState(12)).astype(np.float32)
    fk.set_paths(p0)
    o.paths[...] = p0.reshape(o.paths.shape)
    for _ in range(2):
        fk.run(2)
        o.run()
        assert np.array_equal(_masked(o.ranlux_tab), _masked(fk.bufs[-2]))
        assert np.array_equal(_masked(o.group_tab), _masked(fk.bufs[-1]))
        assert np.array_equal(o.accepts.reshape(-1), fk.bufs[1].reshape(-1))
        assert np.array_equal(o.paths.reshape(-1), fk.bufs[0].reshape(-1))
        ops = fk.bufs[2].reshape(-1)
        assert np.array_equal(o.op_means.reshape(-1)[:ops.size], ops)
    assert fk.bufs[1].sum() > 0


@pytest.mark.parametrize("n,global_path,double", [(10, True, False), (5, False, False), (10, True, True)],
                         ids=["10_atoms_global", "5_atoms_local", "10_atoms_global_fp64"])
def test_oracle_against_live_reference_large_clusters(n, global_path, double):
    """Larger clusters of the generated LM2M2 plugin (the precision study's 10 atoms, 27 DOF,
    45 pairs, global paths, also in the reference's FP64 build; 5 atoms with the path in
    __local memory) against the reference's own kernel (work-groups as fibers, IEEE flags),
    RANLUX, 2 launches: tables, accepts, paths and operator sums bit-exact with the oracle in
    the reference-compatible mode."""
    from oracle import build_ref as br
    if not br.reference_available():
        pytest.skip("reference tree not present")
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    from oracle import ref_timing
    from oracle.oracle import OracleConfig, OracleSampler
    sysm = Lm2m2Cluster(n, 0.7)
    W, N, S = 2, 32, 2
    ka = dict(nbrOfWalkers=W, N=N, beta=float(sysm.beta), S=S, enableOperator=True,
              enableCorrelator=False, enableBisection=True, enablePathShift=False,
              enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
              enableParallelizePath=True, enableGlobalPath=global_path, enableGlobalOldPath=False,
              enableDouble=double, enableRanlux=True, luxuaryFactor=1, ranluxIntMax=2 ** 32 - 1,
              operators=(sysm.energyOp, sysm.meanSquaredRadiusOp), operatorRuns=2, metroStepsPerOperatorRun=2)
    name = f"test_cluster{n}{'_fp64' if double else ''}"
    ref_timing.prepare(name, sysm, ka)
    fk = ref_timing.FiberKernel(name, fast=False)
    o = OracleSampler(OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=W, N=N,
        beta=ka["beta"], S=S, operatorRuns=2, metroStepsPerOperatorRun=2, nbrOfWalkersPerWorkGroup=1,
        enableParallelizePath=True, enableRanlux=True, luxuaryFactor=1, ranluxIntMax=2 ** 32 - 1,
        enableDouble=double, operators=(sysm.energyOp, sysm.meanSquaredRadiusOp), compat=True, accum=0))
    fk.init_ranlux(2)
    o.ranlux_tab[...] = fk.bufs[-2].reshape(o.ranlux_tab.shape)
    o.group_tab[...] = fk.bufs[-1].reshape(o.group_tab.shape)
    p0 = sysm.initial_paths(W, N, np.random.RandomState(n)).astype(np.float64 if double else np.float32)
    fk.set_paths(p0)
    o.paths[...] = p0.reshape(o.paths.shape)
    for _ in range(2):
        fk.run(2)
        o.run()
        assert np.array_equal(_masked(o.ranlux_tab), _masked(fk.bufs[-2]))
        assert np.array_equal(o.accepts.reshape(-1), fk.bufs[1].reshape(-1))
        assert np.array_equal(o.paths.reshape(-1), fk.bufs[0].reshape(-1))
        ops = fk.bufs[2].reshape(-1)
        assert np.array_equal(o.op_means.reshape(-1)[:ops.size], ops)
    assert fk.bufs[1].sum() > 0


def test_oracle_against_live_reference_ho_bench_configuration():
    """The harmonic oscillator's benchmarked configuration against the reference's own kernel:
    xorshift, N = 128, S = 3, the path in __local memory (work-groups as fibers), x^2 and the
    correlator every sweep (a work-group barrier per lag and slice, kernel.c:792), 2 launches
    of 3 sweeps; the oracle in the reference-compatible mode on the same seed table: seed
    rows, accept counts, paths, operator and correlator sums bit-exact.  One walker, i.e. one
    work-group: every work-item reads the shared offset-seed row at its start and writes it
    at its end (kernel.c:568-572, :832-835), so work-groups that run one after another see
    each other's writes, which the oracle's all-read-then-all-write order does not model."""
    from oracle import build_ref as br
    if not br.reference_available():
        pytest.skip("reference tree not present")
    from feynsimul_gb300.physical_systems.harm_osc import HarmOsc
    from oracle import ref_timing
    from oracle.oracle import OracleConfig, OracleSampler
    sysm = HarmOsc()
    ka = dict(nbrOfWalkers=1, N=128, beta=10.0, S=3, enableOperator=True, enableCorrelator=True,
              enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
              nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
              enableGlobalOldPath=False, enableDouble=False, enableRanlux=False,
              operators=(sysm.energyOp,), correlators=("x1",), operatorRuns=3, metroStepsPerOperatorRun=1)
    ref_timing.prepare("test_ho_bench", sysm, ka)
    fk = ref_timing.FiberKernel("test_ho_bench", fast=False)
    o = OracleSampler(OracleConfig(
        DOF=1, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=1, N=128, beta=10.0, S=3,
        operatorRuns=3, metroStepsPerOperatorRun=1, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True,
        operators=(sysm.energyOp,), correlators=("x1",), compat=True, accum=0))
    paths, accepts, seeds, ops, cors = fk.bufs
    o.seeds[...] = seeds.reshape(o.seeds.shape)
    p0 = (np.random.RandomState(13).randn(1, 128) * 0.6).astype(np.float32)
    fk.set_paths(p0)
    o.paths[...] = p0.reshape(o.paths.shape)
    for _ in range(2):
        fk.run(2)
        o.run()
        assert np.array_equal(o.seeds.reshape(-1), seeds.reshape(-1))
        assert np.array_equal(o.accepts.reshape(-1), accepts.reshape(-1))
        assert np.array_equal(o.paths.reshape(-1), paths.reshape(-1))
        assert np.array_equal(o.op_means.reshape(-1)[:ops.size], ops.reshape(-1))
        assert np.array_equal(o.cor_means.reshape(-1), cors.reshape(-1))
    assert accepts.sum() > 0


@pytest.mark.parametrize("case", ["xorshift_walker", "xorshift_parallel"])
def test_oracle_study_correlator_columns(case):
    """Precision-study accumulation sums the same products three ways on one trajectory:
    its FP64 column (float-float per measurement, then FP64) equals the FP64 mode's sums bit
    for bit, and in walker mode (where the FP32 mode also adds slices in ascending order) its
    plain-FP32 column equals the FP32 mode's sums bit for bit; the Kahan column lies between
    in error."""
    ka, _ = load_sweep(case)
    rng = np.random.RandomState(5)
    outs = {}
    for accum in (0, 1, 3):
        o = orc.OracleSampler(oracle_config(ka, compat=False, accum=accum))
        if accum == 0:
            p0 = (rng.randn(*o.paths.shape) * 0.4).astype(o.paths.dtype)
            s0 = rng.randint(0, 2 ** 31 - 1, size=o.seeds.shape).astype(np.uint32)
            w0 = rng.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape).astype(np.uint32)
        o.paths[...] = p0
        o.seeds[...] = s0
        o.walker_seeds[...] = w0
        for _ in range(3):
            o.run()
        outs[accum] = o
    st = outs[3].cor_means
    assert np.array_equal(outs[3].paths, outs[1].paths)
    assert np.array_equal(st["d"], outs[1].cor_means)
    if not ka["enableParallelizePath"]:
        assert np.array_equal(st["f"], outs[0].cor_means)
    ref = st["d"]
    err_f = np.abs(st["f"].astype(np.float64) - ref).max()
    err_k = np.abs(st["ks"].astype(np.float64) - ref).max()
    assert err_k <= err_f + 1e-12
    assert err_f <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("parallel", [True, False], ids=["parallel", "walker"])
def test_oracle_correlator_sums_against_exact(parallel):
    """One sweep, then one measurement: each lag's correlator sum comes from the final path
    alone, so it is checked against the exact sum (math.fsum) of the same FP32 products.
    The FP64 column (float-float per measurement, then FP64) stays within N * 2^-48 * sum|q|
    of it; the plain FP32 column is typically ~1e3 times further off."""
    import math
    W, N, S = 8, 64, 3
    cfg = orc.OracleConfig(DOF=1, potential=HO["potential"], userCode=HO["userCode"], nbrOfWalkers=W, N=N,
                           beta=10.0, S=S, operatorRuns=1, metroStepsPerOperatorRun=1,
                           enableParallelizePath=parallel, operators=("x1 * x1",), correlators=("x1",),
                           accum=3)
    o = orc.OracleSampler(cfg)
    rng = np.random.RandomState(11)
    o.paths[...] = (rng.randn(*o.paths.shape) * 10 ** rng.uniform(-2, 2, size=o.paths.shape)).astype(np.float32)
    o.seeds[...] = rng.randint(0, 2 ** 31 - 1, size=o.seeds.shape).astype(np.uint32)
    o.walker_seeds[...] = rng.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape).astype(np.uint32)
    o.run()
    x = o.paths.reshape(W, N).astype(np.float32)
    st = o.cor_means.reshape(W, N // 2)
    worst_d = worst_f = 0.0
    for w in range(W):
        for tau in range(N // 2):
            q = (x[w] * np.roll(x[w], -tau)).astype(np.float64)   # FP32 products, exactly in FP64
            exact = math.fsum(q)
            scale = float(np.abs(q).sum())
            assert abs(st["d"][w, tau] - exact) <= N * 2.0 ** -48 * scale
            worst_d = max(worst_d, abs(st["d"][w, tau] - exact) / scale)
            worst_f = max(worst_f, abs(float(st["f"][w, tau]) - exact) / scale)
    assert worst_d < 1e-3 * worst_f


def _golden_lm2m2():
    import os
    from golden_cases import GOLDEN
    z = np.load(os.path.join(GOLDEN, "lm2m2_ref.npz"))
    return {k: z[k] for k in z.files}


def test_lm2m2_numpy_matches_reference_header():
    """The LM2M2 restatement against the reference's lm2m2.h built as-is (golden)."""
    from feynsimul_gb300.physical_systems.lm2m2 import lm2m2_numpy
    g = _golden_lm2m2()
    r = np.sqrt(g["r2_double"])
    v, dv_ref_form = lm2m2_numpy(r, reference_derivative=True)
    np.testing.assert_allclose(v, g["v_double"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(dv_ref_form, g["dv_double"], rtol=1e-12, atol=1e-12)
    # the correct derivative equals d/d(r^2) of the potential (numerically)
    _, dv = lm2m2_numpy(r)
    r2, h = g["r2_double"], 1e-6 * g["r2_double"]
    num = (lm2m2_numpy(np.sqrt(r2 + h))[0] - lm2m2_numpy(np.sqrt(r2 - h))[0]) / (2 * h)
    np.testing.assert_allclose(dv, num, rtol=1e-5, atol=1e-8)


def _plugin_c_lib(code, ft):
    import ctypes
    import hashlib
    import os
    import subprocess
    import tempfile
    src = ("#include <tgmath.h>\n#define FLOAT_TYPE %s\n#define rsqrt(x) (1 / sqrt(x))\n%s\n"
           "void eval(const FLOAT_TYPE *r2, FLOAT_TYPE *v, FLOAT_TYPE *dv, int n)\n"
           "{ for (int i = 0; i < n; i++) { v[i] = lm2m2_r2(r2[i]); dv[i] = dlm2m2_dr2(r2[i]); } }\n") % (ft, code)
    d = tempfile.mkdtemp(prefix="fs_lm2m2_")
    h = hashlib.sha1(src.encode()).hexdigest()[:12]
    c, so = os.path.join(d, f"p{h}.c"), os.path.join(d, f"p{h}.so")
    open(c, "w").write(src)
    flags = ["-std=gnu11", "-O2", "-ffp-contract=off", "-fgnu89-inline", "-fPIC", "-shared", "-w"]
    if ft == "float":
        flags.append("-fsingle-precision-constant")
    subprocess.run(["gcc", *flags, c, "-o", so, "-lm"], check=True)
    lib = ctypes.CDLL(so)
    lib.eval.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
    return lib


@pytest.mark.parametrize("branchless", [True, False])
@pytest.mark.parametrize("reference_derivative", [False, True])
def test_lm2m2_plugin_code_matches_restatement(branchless, reference_derivative):
    """The plugin's C code (as pasted into the sweep kernel) against the numpy restatement,
    in FP64 to 1e-12 and in FP32 to FP32 rounding."""
    from feynsimul_gb300.physical_systems.lm2m2 import lm2m2_c_code, lm2m2_numpy
    g = _golden_lm2m2()
    code = lm2m2_c_code(reference_derivative, branchless=branchless)
    r2 = np.ascontiguousarray(g["r2_double"])
    want_v, want_dv = lm2m2_numpy(np.sqrt(r2), reference_derivative=reference_derivative)
    lib = _plugin_c_lib(code, "double")
    v, dv = np.zeros_like(r2), np.zeros_like(r2)
    lib.eval(r2.ctypes.data, v.ctypes.data, dv.ctypes.data, len(r2))
    np.testing.assert_allclose(v, want_v, rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(dv, want_dv, rtol=1e-11, atol=1e-11)
    r2f = np.ascontiguousarray(r2.astype(np.float32))
    libf = _plugin_c_lib(code, "float")
    vf, dvf = np.zeros_like(r2f), np.zeros_like(r2f)
    libf.eval(r2f.ctypes.data, vf.ctypes.data, dvf.ctypes.data, len(r2f))
    # FP32: the repulsive and dispersion terms cancel near r_m, so the error is relative
    # to the terms (a few K there), not to V
    assert np.all(np.abs(vf - want_v) <= 2e-6 * np.abs(want_v) + 5e-4)
    sel = np.sqrt(r2) > 2.2
    np.testing.assert_allclose(dvf[sel], want_dv[sel], rtol=1e-4, atol=5e-3)
