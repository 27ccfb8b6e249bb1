"""The C-ABI boundary without a GPU: the library builds for sm_103a, loads, exports every
symbol include/feynsimul.h declares, and the NVRTC path compiles plugin code (the OpenCL
spellings and single-precision literals of the reference's plugins) for sm_103a."""
import ctypes
import os
import re
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from feynsimul_gb300 import build, _lib
    build.build()
    return _lib


def header_symbols():
    text = open(os.path.join(ROOT, "include", "feynsimul.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fs_[a-z0-9_]+)\s*\(", text)))


def test_exports_match_header():
    L = _lib()
    syms = header_symbols()
    assert set(syms) == set(L.EXPORTS)
    so = ctypes.CDLL(L.LIB_PATH)
    for s in syms:
        assert hasattr(so, s), s
    assert b"sm_103a" in L.lib().fs_version()


def _cfg(**kw):
    import __graft_entry__ as g
    return g._ho_config(**kw)


def _compile(cfg, pot, uc="", ops=(), cors=(), hists=()):
    L = _lib()
    o, no = L.strings(ops)
    c, nc = L.strings(cors)
    h, nh = L.strings(hists)
    buf = ctypes.create_string_buffer(1 << 16)
    rc = L.lib().fs_compile_only(ctypes.byref(cfg), pot.encode(), uc.encode(), o, no, c, nc, h, nh,
                                 buf, len(buf))
    return rc, buf.value.decode(errors="replace")


@pytest.mark.parametrize("kw", [
    dict(),
    dict(enable_ranlux=1, compat=1, accum=0, fast_math=0, enable_bins=1),
    dict(enable_parallelize_path=0, walkers_per_group=1),
    dict(enable_double=1, accum=3),
    dict(n_slices=2048, bisection_level=2, n_walkers=4),   # 512 threads per walker
    dict(partials=1),                                       # exact partials
    dict(accum=2),                                          # Kahan operators, pipelined lags
    dict(accum=2, enable_parallelize_path=0, walkers_per_group=1),  # FMA partials, one lag loop
    dict(n_slices=2, bisection_level=1),                    # N not a multiple of 4
    dict(potential_cache=3),                                # potential cache in device memory
    dict(potential_cache=3, enable_parallelize_path=0, walkers_per_group=1, enable_ranlux=1),
    dict(potential_cache=3, global_path=1, enable_double=1),
])
def test_nvrtc_compiles_for_sm103a(kw):
    rc, log = _compile(_cfg(**kw), "0.5 * 1.0 * x1 * x1", "FLOAT_TYPE sqr(FLOAT_TYPE x){return x*x;}",
                       ("1.0 * x1 * x1", "native_exp(-sqr(x1))"), ("x1",))
    assert rc == 0, log
    assert "fs_metropolis" in log


def test_nvrtc_compiles_five_correlators():
    # the pipelined lag sums of more correlators than fit in registers (running sums in
    # device memory)
    rc, log = _compile(_cfg(), "0.5 * 1.0 * x1 * x1", "", ("1.0 * x1 * x1",),
                       ("x1", "x1 * x1", "x1 * x1 * x1", "0.5 * x1", "x1 - 1.0"))
    assert rc == 0, log


@pytest.mark.parametrize("N,S,W,ncor,accum", [
    (16, 1, 32, 1, 1), (16, 2, 8, 2, 1), (32, 3, 64, 1, 2), (64, 1, 64, 1, 1), (64, 2, 33, 1, 1),
    (64, 3, 128, 3, 1), (128, 2, 64, 1, 1), (128, 3, 1024, 2, 0), (128, 4, 96, 1, 3), (256, 2, 32, 1, 1),
    (256, 3, 64, 5, 1), (512, 4, 32, 1, 1), (1024, 5, 16, 1, 1), (64, 6, 64, 1, 1), (32, 5, 32, 1, 1),
])
def test_correlator_launch_shapes_compile(N, S, W, ncor, accum):
    # the host's choice of correlator helpers (after the moves, pipelined, or none) and lag
    # layout for a spread of shapes, walker counts, correlator counts and accumulations
    rc, log = _compile(_cfg(n_slices=N, bisection_level=S, n_walkers=W, accum=accum),
                       "0.5 * x1 * x1", "", ("x1 * x1",), tuple("x1" + " * x1" * k for k in range(ncor)))
    assert rc == 0, log


def test_lm2m2_plugin_compiles():
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    s = Lm2m2Cluster(4, 0.5)
    rc, log = _compile(_cfg(dof=s.DOF, n_slices=64, bisection_level=3, beta=s.beta, enable_ranlux=1,
                            hist_lo=0.0, hist_hi=20.0, hist_bins=200),
                       s.potential, s.userCode, (s.energyOp, s.meanSquaredRadiusOp), (), s.pairDistanceOps)
    assert rc == 0, log


def test_compile_error_is_reported():
    rc, log = _compile(_cfg(), "0.5 * x1 * undefined_thing")
    assert rc == -2 and "undefined_thing" in log


@pytest.mark.parametrize("kw,msg", [
    (dict(n_slices=100), "power of 2"),
    (dict(bisection_level=9), "2^S"),
    (dict(n_walkers=10, walkers_per_group=4), "multiple"),
    (dict(enable_ranlux=1, luxury_factor=7), "luxuaryFactor"),
    (dict(potential_cache=4), "potential_cache"),
])
def test_config_errors(kw, msg):
    rc, log = _compile(_cfg(**kw), "x1")
    assert rc == -1 and msg in log


def test_mlp_train_step_rejects_misaligned_buffers():
    # checked before any device work: the pointers are never dereferenced
    L = _lib()
    rc = L.lib().fs_mlp_train_step(ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1002), ctypes.c_void_p(0x2000),
                                   ctypes.c_void_p(0x3000), ctypes.c_void_p(0x4000), 128, 6,
                                   ctypes.c_float(1.0 / 128), None, None)
    assert rc == L.FS_ERR_CONFIG
    assert b"16-byte aligned" in L.lib().fs_last_error(None)


def test_python_validation_matches_reference_messages():
    from feynsimul_gb300.kernel import PIMCKernel
    from feynsimul_gb300.kernel_args import KernelArgs
    sysm = types.SimpleNamespace(DOF=1, potential="x1*x1", userCode="")
    base = dict(system=sysm, nbrOfWalkers=4, N=16, beta=1.0, S=2, enableOperator=False,
                enableCorrelator=False, enableBisection=True, enablePathShift=False,
                enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
                enableParallelizePath=True, enableGlobalPath=False, enableGlobalOldPath=False,
                operatorRuns=1, metroStepsPerOperatorRun=1)
    with pytest.raises(TypeError, match="beta need to be a float"):
        PIMCKernel(KernelArgs(**dict(base, beta=1)))
    with pytest.raises(Exception, match="power of 2"):
        PIMCKernel(KernelArgs(**dict(base, N=12)))
    with pytest.raises(NameError, match="operators need to be set"):
        PIMCKernel(KernelArgs(**dict(base, enableOperator=True)))
    with pytest.raises(Exception, match="Single node move not possible"):
        PIMCKernel(KernelArgs(**dict(base, enableSingleNodeMove=True, alpha=0.1)))


def test_float_literal_rewrite_in_generated_source():
    rc, log = _compile(_cfg(), "0.5 * x1 * x1 + 1e-3 + 2. * .25 + 0x1p-3")
    assert rc == 0, log


def test_c_caller_links_and_compiles_a_sweep(tmp_path):
    """tests/c/abi_check.c: the header and library used from C, as any FFI would."""
    import shutil
    import subprocess
    L = _lib()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_check")
    libdir = os.path.dirname(L.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_check.c"), "-L", libdir, "-lfeynsimul_gb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    env = dict(os.environ, FS_CACHE_DIR=str(tmp_path / "cache"))
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and "abi ok" in r.stdout, r.stdout + r.stderr


def test_ctypes_structs_match_the_c_header(tmp_path):
    """The Python mirrors of the C ABI's structs (feynsimul_gb300/_lib.py) have the header's
    size and member offsets (tests/c/abi_layout.c prints them as the C compiler lays them out)."""
    import shutil
    import subprocess
    L = _lib()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_layout")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_layout.c"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    mirrors = {"fs_config": L.FsConfig, "fs_info": L.FsInfo, "fs_batch_system": L.FsBatchSystem}
    seen = {k: set() for k in mirrors}
    for line in filter(None, out):
        struct, member, value = line.split()
        cls = mirrors[struct]
        if member == "sizeof":
            assert ctypes.sizeof(cls) == int(value), struct
        else:
            assert getattr(cls, member).offset == int(value), (struct, member)
            seen[struct].add(member)
    for struct, cls in mirrors.items():
        assert seen[struct] == {f[0] for f in cls._fields_}, struct   # every member, both sides
