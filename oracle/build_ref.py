"""Build recipe for ``oracle/_ref``: the reference's own OpenCL C compiled on the CPU.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``tests/golden/make_golden.py`` and the
oracle may use this module; the product never does.  It needs the reference's source tree
(``REFERENCE_ROOT``: the ``FEYNSIMUL_REFERENCE_ROOT`` environment variable, else the
development container's mount); everything it builds goes to ``oracle/_ref/`` (git-ignored).  Where
the tree is absent nothing here runs: the goldens it produces are committed under
``tests/golden/``.

What it does:

* imports the reference's ``FeynSimul/kernel.py`` (Python 2 era code that still parses as
  Python 3) with a stub ``pyopencl`` package that records the OpenCL program text instead
  of compiling it, so the kernel source is produced by the reference's own substitution
  rules (kernel.py:215-348) and its own seed tables (kernel.py:396-426);
* compiles that text plus the vendored RANLUXCL header (examples/pyopencl-ranluxcl.cl)
  with gcc through ``oracle/cl_shim.h`` into a shared object with a small NDRange
  launcher (one POSIX thread per work-item, see cl_shim.h for the barrier model);
* runs ``metropolis`` / ``ranlux_init_kernel`` / ``ranlux_group_init_kernel`` on numpy
  buffers, and dumps RANLUXCL uniform streams for every luxury level.

The one textual change applied to the generated text (never to the reference files) is
the OpenCL swizzle ``(*seedPtr).xyz=(*seedPtr).yzw;`` (kernel.c:218), which has no C
spelling; it is replaced by the three equivalent scalar assignments.
"""
from __future__ import annotations

import contextlib
import ctypes
import hashlib
import os
import subprocess
import sys
import types

import numpy as np

# The reference's source tree: the FEYNSIMUL_REFERENCE_ROOT environment variable, else the
# read-only mount this recipe was written for.
REFERENCE_ROOT = os.environ.get("FEYNSIMUL_REFERENCE_ROOT") or "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, "_ref")

SWIZZLE = "(*seedPtr).xyz=(*seedPtr).yzw;"
SWIZZLE_C = ("{ uint4 _fs_t = *seedPtr; (*seedPtr).x = _fs_t.y; "
             "(*seedPtr).y = _fs_t.z; (*seedPtr).z = _fs_t.w; }")

CFLAGS = ["-std=gnu11", "-O2", "-fsingle-precision-constant", "-ffp-contract=off",
          "-fgnu89-inline", "-fPIC", "-shared", "-Wno-unknown-pragmas", "-w"]


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "FeynSimul", "kernel.py"))


# --------------------------------------------------------------------------------------
# stub pyopencl: records what kernel.py asks OpenCL to do
# --------------------------------------------------------------------------------------
class _StubArray:
    def __init__(self, arr):
        self.arr = arr
        self.data = self

    def get(self):
        return self.arr.copy()


def _shape(s):
    if isinstance(s, (tuple, list)):
        return tuple(int(v) for v in s)
    return (int(s),)


class _StubProgram:
    last = None

    def __init__(self, ctx, source):
        self.source = source
        self.options = None
        _StubProgram.last = self

    def build(self, options=None):
        self.options = options
        return self

    def __getattr__(self, name):  # prg.metropolis, prg.ranlux_init_kernel, ...
        if name.startswith("__"):
            raise AttributeError(name)
        return name


def _install_stub_pyopencl():
    if "pyopencl" in sys.modules and not getattr(sys.modules["pyopencl"], "_fs_stub", False):
        raise RuntimeError("a real pyopencl is imported; the stub cannot be installed")
    cl = types.ModuleType("pyopencl")
    cl._fs_stub = True
    cl.create_some_context = lambda *a, **k: object()
    cl.command_queue_properties = types.SimpleNamespace(PROFILING_ENABLE=1)
    cl.CommandQueue = lambda *a, **k: types.SimpleNamespace(finish=lambda: None)
    cl.Program = _StubProgram
    cl.MemoryError = MemoryError
    cl.RuntimeError = RuntimeError
    arr = types.ModuleType("pyopencl.array")
    arr.zeros = lambda q, shape, dtype: _StubArray(np.zeros(_shape(shape), dtype))
    arr.to_device = lambda q, a: _StubArray(np.array(a, copy=True))
    cl.array = arr
    sys.modules["pyopencl"] = cl
    sys.modules["pyopencl.array"] = arr
    for sub in ("clrandom", "clmath"):
        m = types.ModuleType("pyopencl." + sub)
        setattr(cl, sub, m)
        sys.modules["pyopencl." + sub] = m


@contextlib.contextmanager
def _int_sizes_randint():
    """Under Python 3 division kernel.py computes some array sizes as floats
    (kernel.py:200-207 feeding :402, :408, :417-420); cast them to int."""
    orig_randint, orig_zeros = np.random.randint, np.zeros

    def randint(low, high=None, size=None, dtype=int):
        if size is not None:
            size = _shape(size)
        return orig_randint(low, high=high, size=size, dtype=dtype)

    def zeros(shape, dtype=float, *a, **k):
        return orig_zeros(_shape(shape), dtype, *a, **k)

    np.random.randint, np.zeros = randint, zeros
    try:
        yield
    finally:
        np.random.randint, np.zeros = orig_randint, orig_zeros


def reference_modules():
    """Import the reference's kernel/kernel_args modules with the stub pyopencl."""
    if not reference_available():
        raise RuntimeError("reference tree not present")
    _install_stub_pyopencl()
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import FeynSimul.kernel as rk  # noqa: E402
    import FeynSimul.kernel_args as rka  # noqa: E402
    return rk, rka


def capture(ka_kwargs: dict, system, np_seed: int):
    """Run the reference's PIMCKernel.__init__ under the stub; return what it produced."""
    rk, rka = reference_modules()
    ka = rka.KernelArgs(system=system, **ka_kwargs)
    # kernel_args.py takes PSAlpha (:41) but never stores it, and kernel.py:127 reads
    # ka.PSAlpha: set the attribute as a caller of the reference has to
    if "PSAlpha" in ka_kwargs and not hasattr(ka, "PSAlpha"):
        ka.PSAlpha = ka_kwargs["PSAlpha"]
    np.random.seed(np_seed)
    with _int_sizes_randint():
        k = rk.PIMCKernel(ka)
    prg = _StubProgram.last
    out = {
        "source": prg.source,
        "options": prg.options,
        "global_size": tuple(int(v) for v in k._globalSize),
        "local_size": None if k._localSize is None else tuple(int(v) for v in k._localSize),
        "n_threads": int(k._nbrOfThreads),
        "kernel": k,
    }
    return out


# --------------------------------------------------------------------------------------
# compile + launch
# --------------------------------------------------------------------------------------
def _compile(tag_text: str, c_text: str, name: str, single_constants: bool = True) -> str:
    os.makedirs(REF_BUILD, exist_ok=True)
    flags = [f for f in CFLAGS if single_constants or f != "-fsingle-precision-constant"]
    with open(os.path.join(HERE, "cl_shim.h")) as f:
        shim = f.read()
    h = hashlib.sha1((tag_text + c_text + " ".join(flags) + shim).encode()).hexdigest()[:16]
    so = os.path.join(REF_BUILD, f"{name}_{h}.so")
    if os.path.exists(so):
        return so
    src = os.path.join(REF_BUILD, f"{name}_{h}.c")
    with open(src, "w") as f:
        f.write(c_text)
    cmd = ["gcc", *flags, "-I", HERE, "-I", os.path.join(REFERENCE_ROOT, "examples"),
           src, "-o", so + ".tmp", "-lpthread", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
    os.replace(so + ".tmp", so)
    return so


_LAUNCHER = r"""
/* NDRange launcher for the reference kernels (oracle/_ref; test infrastructure). */
_Thread_local clsh_item_t clsh_item;
pthread_barrier_t *clsh_barrier;
typedef struct { clsh_item_t item; void **a; int which; } clsh_job_t;
static void *clsh_work(void *p)
{
    clsh_job_t *j = (clsh_job_t *)p;
    clsh_item = j->item;
    void **a = j->a;
    (void)a;
    switch (j->which) {
    case 0: metropolis(%(METRO_ARGS)s); break;
%(RANLUX_CASES)s
    }
    return 0;
}
int clsh_launch(int which, void **a, size_t g0, size_t g1, size_t l0, size_t l1)
{
    size_t n = g0 * g1, i;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, 0, (unsigned)n);
    clsh_barrier = &bar;
    pthread_t *th = (pthread_t *)calloc(n, sizeof(pthread_t));
    clsh_job_t *jobs = (clsh_job_t *)calloc(n, sizeof(clsh_job_t));
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, 1 << 20);
    for (i = 0; i < n; i++) {
        size_t i0 = i %% g0, i1 = i / g0;
        clsh_item_t it = {{i0, i1, 0}, {i0 %% l0, i1 %% l1, 0}, {i0 / l0, i1 / l1, 0},
                          {g0, g1, 1}, {l0, l1, 1}};
        jobs[i].item = it; jobs[i].a = a; jobs[i].which = which;
        if (pthread_create(&th[i], &attr, clsh_work, &jobs[i]) != 0) return -1;
    }
    for (i = 0; i < n; i++) pthread_join(th[i], 0);
    pthread_barrier_destroy(&bar);
    free(th); free(jobs);
    return 0;
}
"""


def kernel_buffers(k):
    """The metropolis kernel's buffers in argument order (the reference kernel's own numpy
    arrays behind kernel.py's stub buffers), the C casts of the launcher's argument list, and
    the launcher cases of the RANLUX initialisation kernels."""
    ft = "double" if k._enableDouble else "float"
    args = []

    def add(cast):
        args.append(f"({cast})a[{len(args)}]")

    bufs = [k._paths, k._accepts]
    add(f"{ft} *"); add("uint *")
    if not k._enableRanlux:
        bufs.append(k._seeds); add("uint *")
    if k._enableGlobalOldPath:
        bufs.append(k._oldPath); add(f"{ft} *")
    if k._enableOperator:
        bufs.append(k._operatorValues); add(f"{ft} *")
    if k._enableCorrelator:
        bufs.append(k._correlatorValues); add(f"{ft} *")
    if k._enableBins:
        bufs.append(k._binCounts); add("uint *")
    ranlux_cases = ""
    if k._enableRanlux:
        bufs += [k._ranluxcltab, k._groupRanluxcltab]
        add("ranluxcl_state_t *"); add("ranluxcl_state_t *")
        ranlux_cases = ("    case 1: ranlux_init_kernel((uint *)a[0], (ranluxcl_state_t *)a[1]); break;\n"
                        "    case 2: ranlux_group_init_kernel((uint *)a[0], (ranluxcl_state_t *)a[1]); break;\n")
    return bufs, args, ranlux_cases


class RefKernel:
    """The reference's metropolis kernel, compiled for the CPU, behind kernel.py's buffers."""

    def __init__(self, ka_kwargs: dict, system, np_seed: int = 0):
        cap = capture(ka_kwargs, system, np_seed)
        k = cap["kernel"]
        self.k = k
        self.parallel = bool(k._enableParallelizePath)
        if self.parallel and not k._enableGlobalPath:
            raise ValueError("the CPU reference build runs parallel-path mode with "
                             "enableGlobalPath=True (no __local memory on the host)")
        self.g = cap["global_size"]
        if cap["local_size"] is None:
            # Walker mode leaves the local size to the OpenCL implementation
            # (kernel.py:209-210).  The compatible definition used throughout this
            # project is a local size of 1.
            self.g = (self.g[0], 1)
            self.l = (1, 1)
        else:
            self.l = cap["local_size"]
        self.bufs, args, ranlux_cases = kernel_buffers(k)
        src = cap["source"].replace(SWIZZLE, SWIZZLE_C)
        launcher = _LAUNCHER % {"METRO_ARGS": ", ".join(args), "RANLUX_CASES": ranlux_cases}
        c_text = ('#include "cl_shim.h"\n#include <stdlib.h>\n' + src + "\n" + launcher)
        # kernel.py:376-377: single-precision constants unless enableDouble
        self.so_path = _compile("metropolis", c_text, "metropolis",
                                single_constants=not k._enableDouble)
        self.lib = ctypes.CDLL(self.so_path)
        self.lib.clsh_launch.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.c_size_t, ctypes.c_size_t,
                                         ctypes.c_size_t, ctypes.c_size_t]
        self.lib.clsh_launch.restype = ctypes.c_int
        self.source = src

    # buffers are the reference kernel's own numpy arrays (k._paths.arr, ...)
    def _launch(self, which, arrays):
        for a in arrays:
            assert a.flags["C_CONTIGUOUS"]
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        rc = self.lib.clsh_launch(which, ptrs, self.g[0], self.g[1], self.l[0], self.l[1])
        if rc != 0:
            raise RuntimeError("thread creation failed")

    def run(self):
        self._launch(0, [b.arr for b in self.bufs])

    def init_ranlux(self):
        self._launch(1, [self.k._seeds.arr, self.k._ranluxcltab.arr])

    def group_init_ranlux(self):
        self._launch(2, [self.k._groupSeeds.arr, self.k._groupRanluxcltab.arr])

    def set_paths(self, paths):
        a = np.ascontiguousarray(paths, dtype=self.k._paths.arr.dtype)
        self.k._paths.arr[...] = a.reshape(self.k._paths.arr.shape)


# --------------------------------------------------------------------------------------
# RANLUXCL stream dumps (the vendored header compiled as-is)
# --------------------------------------------------------------------------------------
_RANLUX_DUMP = r"""
#define RANLUXCL_LUX %(LUX)d
#include "pyopencl-ranluxcl.cl"
_Thread_local clsh_item_t clsh_item;
pthread_barrier_t *clsh_barrier;
/* seed one state exactly as ranluxcl_init does (pyopencl-ranluxcl.cl:597-725) */
void ref_ranlux_init(unsigned long x, ranluxcl_state_t *st) { ranluxcl_init(x, st); }
/* n_calls consecutive ranluxcl32 calls -> 4*n_calls floats */
void ref_ranlux_stream(ranluxcl_state_t *st, float *out, int n_calls)
{
    int i;
    for (i = 0; i < n_calls; i++) {
        float4 v = ranluxcl32(st);
        out[4 * i + 0] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
    }
}
void ref_ranlux_stream64(ranluxcl_state_t *st, double *out, int n_calls)
{
    int i;
    for (i = 0; i < n_calls; i++) {
        double4 v = ranluxcl64(st);
        out[4 * i + 0] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
    }
}
"""


def ranlux_dump_lib(lux: int):
    c_text = ('#include "cl_shim.h"\n#define RANLUXCL_SUPPORT_DOUBLE\n'
              + _RANLUX_DUMP % {"LUX": lux})
    lib = ctypes.CDLL(_compile(f"lux{lux}", c_text, f"ranlux_lux{lux}"))
    lib.ref_ranlux_init.argtypes = [ctypes.c_ulong, ctypes.c_void_p]
    lib.ref_ranlux_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.ref_ranlux_stream64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    return lib


def ref_ranlux_streams(lux: int, seeds, n_calls: int, double=False):
    """Return (streams[n_seeds, 4*n_calls], final states[n_seeds, 28] as uint32)."""
    lib = ranlux_dump_lib(lux)
    seeds = [int(s) for s in seeds]
    out = np.zeros((len(seeds), 4 * n_calls), np.float64 if double else np.float32)
    states = np.zeros((len(seeds), 28), np.uint32)
    for i, s in enumerate(seeds):
        st = np.zeros(28, np.uint32)
        lib.ref_ranlux_init(s, st.ctypes.data)
        row = np.zeros(4 * n_calls, out.dtype)
        if double:
            lib.ref_ranlux_stream64(st.ctypes.data, row.ctypes.data, n_calls)
        else:
            lib.ref_ranlux_stream(st.ctypes.data, row.ctypes.data, n_calls)
        out[i] = row
        states[i] = st
    return out, states


def reference_plugin_values(module: str, cls: str, attrs, x):
    """FP64 values of expression attributes of the reference's plugin class
    physical_systems/<module>.py:<cls> at coordinates x [m, DOF]: the class is instantiated
    from the reference tree and its userCode and expressions are compiled as-is."""
    import importlib.util
    path = os.path.join(REFERENCE_ROOT, "FeynSimul", "physical_systems", module + ".py")
    spec = importlib.util.spec_from_file_location("ref_" + module, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    obj = getattr(mod, cls)()
    dof = int(obj.DOF)
    decl = " ".join(f"double x{k + 1} = x[{k}];" for k in range(dof))
    fns = "".join(f"static double ref_f{i}(const double *x) {{ {decl} return {getattr(obj, a)}; }}\n"
                  for i, a in enumerate(attrs))
    calls = " ".join(f"out[(size_t)r * {len(attrs)} + {i}] = ref_f{i}(x + (size_t)r * {dof});"
                     for i in range(len(attrs)))
    c_text = ('#include "cl_shim.h"\n#define FLOAT_TYPE double\n' + obj.userCode + "\n" + fns +
              "void ref_plugin_eval(const double *x, int m, double *out)\n"
              "{ int r; for (r = 0; r < m; r++) { " + calls + " } }\n")
    lib = ctypes.CDLL(_compile("double", c_text, f"plugin_{module}", single_constants=False))
    lib.ref_plugin_eval.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.shape[0], len(attrs)))
    lib.ref_plugin_eval(x.ctypes.data, x.shape[0], out.ctypes.data)
    return out


def lm2m2_header_lib():
    """The reference's physical_systems/lm2m2.h compiled as-is: lm2m2sqrt / dlm2m2sqrtdr."""
    c_text = ('#include "cl_shim.h"\n#define FLOAT_TYPE %(FT)s\n'
              '#include "' + os.path.join(REFERENCE_ROOT, "FeynSimul", "physical_systems", "lm2m2.h") + '"\n'
              'void ref_lm2m2(const %(FT)s *sr, %(FT)s *v, %(FT)s *dv, int n)\n'
              '{ int i; for (i = 0; i < n; i++) { v[i] = lm2m2sqrt(sr[i]); dv[i] = dlm2m2sqrtdr(sr[i]); } }\n')
    libs = {}
    for ft in ("float", "double"):
        lib = ctypes.CDLL(_compile(ft, c_text % {"FT": ft}, f"lm2m2_{ft}",
                                   single_constants=(ft == "float")))
        lib.ref_lm2m2.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
        libs[ft] = lib
    return libs
