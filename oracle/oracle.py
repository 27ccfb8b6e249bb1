"""CPU oracle driver: builds and runs the C restatement in ``oracle/pimc_oracle.c``.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``, and only as the checker or
the timed CPU baseline -- never by the product package.

The run parameters are derived here independently of the product, following the
reference's kernel.py:
  * launch geometry and thread ids .......... kernel.py:192-211, kernel.c:538-541
  * epsilon / opNorm literals ('%1.17e') .... kernel.py:298, :312-313
  * RANLUX luxury+1, ranluxIntMax+1 ......... kernel.py:132-147, :331-334
  * histogram constants ..................... kernel.py:336-342
  * float constants for FP32 builds ........ kernel.py:376-377 (-cl-single-precision-constant)
Plugin strings are pasted unmodified (C is close enough to OpenCL C for them).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

_NSKIP = {0: 0, 1: 24, 2: 76, 3: 200, 4: 380}


def nskip_for(lux_in_kernel: int) -> int:
    return _NSKIP.get(lux_in_kernel, lux_in_kernel - 24)


# precision-study correlator accumulator: FP64, plain FP32, Kahan sum and compensation
COR_STUDY_DTYPE = np.dtype([("d", np.float64), ("f", np.float32), ("ks", np.float32), ("kc", np.float32),
                            ("pad", np.float32)])


@dataclass
class OracleConfig:
    """The reference's KernelArgs fields that the sweep uses (kernel_args.py:23-51)."""
    DOF: int
    potential: str
    userCode: str
    nbrOfWalkers: int
    N: int
    beta: float
    S: int
    operatorRuns: int
    metroStepsPerOperatorRun: int
    nbrOfWalkersPerWorkGroup: int = 1
    enableParallelizePath: bool = True
    enableRanlux: bool = False
    luxuaryFactor: int = 2
    ranluxIntMax: int = 2 ** 32 - 1
    enableDouble: bool = False
    operators: tuple = ()
    correlators: tuple = ()
    enableBins: bool = False
    xMin: float = 0.0
    xMax: float = 1.0
    binResolutionPerDOF: int = 1
    enableBisection: bool = True
    enablePathShift: bool = False       # walker mode only (kernel.py:192-198)
    enableSingleNodeMove: bool = False
    alpha: float = 0.0                  # single-node move width (kernel_args.py:124-126)
    PSAlpha: float = 0.0                # path-shift width (kernel_args.py:128-131)
    # additions of this project (same meaning as in the CUDA kernels)
    compat: bool = False
    accum: int = 1                      # 0 ref FP32, 1 FP64, 2 Kahan, 3 study
    histograms: tuple = ()              # expressions binned into one shared histogram
    histRange: tuple = (0.0, 1.0)
    histBins: int = 0

    # ---- derived (kernel.py) ----
    @property
    def seg(self):
        return 2 ** self.S

    @property
    def tpw(self):
        return self.N // self.seg if self.enableParallelizePath else 1

    @property
    def n_threads(self):
        return self.nbrOfWalkers * self.tpw

    @property
    def n_wg(self):
        return self.nbrOfWalkers // self.nbrOfWalkersPerWorkGroup

    @property
    def opnorm(self):
        return 1.0 / float(self.operatorRuns * self.N * self.nbrOfWalkers / self.n_threads)


def _defines(c: OracleConfig) -> str:
    ft = "double" if c.enableDouble else "float"
    d = {
        "FS_DOUBLE": int(c.enableDouble), "FS_DOF": c.DOF, "FS_N": c.N, "FS_S": c.S,
        "FS_SEG": c.seg, "FS_TPW": c.tpw, "FS_NWALKERS": c.nbrOfWalkers,
        "FS_WPG": c.nbrOfWalkersPerWorkGroup, "FS_NWG": c.n_wg,
        "FS_PARALLEL": int(bool(c.enableParallelizePath)), "FS_RANLUX": int(bool(c.enableRanlux)),
        "FS_NSKIP": nskip_for(c.luxuaryFactor + 1),
        "FS_RIM": ("%.9E" % (c.ranluxIntMax + 1)) + "f",
        "FS_COMPAT": int(bool(c.compat)), "FS_ACCUM": int(c.accum),
        "FS_NOPS": len(c.operators), "FS_NCOR": len(c.correlators),
        "FS_OPRUNS": c.operatorRuns, "FS_MSTEPS": c.metroStepsPerOperatorRun,
        "FS_EPS": "%1.17e" % (c.beta / float(c.N)),
        "FS_OPNORM": "%1.17e" % c.opnorm,
        "FS_BINS": int(bool(c.enableBins)),
        "FS_NHIST": len(c.histograms) if c.histBins > 0 else 0,
        "FS_BISECT": int(bool(c.enableBisection)),
        "FS_PATH_SHIFT": int(bool(c.enablePathShift)), "FS_SNM": int(bool(c.enableSingleNodeMove)),
        "FS_EPS_INV2": "%1.17e" % ((float(c.N) / c.beta) ** 2),
        "FS_ALPHA": "%1.17e" % c.alpha, "FS_PSALPHA": "%1.17e" % c.PSAlpha,
    }
    if c.enableBins:
        d.update({"FS_XMIN": "%1.17e" % c.xMin, "FS_XMAX": "%1.17e" % c.xMax,
                  "FS_BINRES": c.binResolutionPerDOF,
                  "FS_INVBIN": "%1.17e" % (float(c.binResolutionPerDOF) / float(c.xMax - c.xMin))})
    if d["FS_NHIST"]:
        lo, hi = c.histRange
        d.update({"FS_HLO": "%1.17e" % lo, "FS_HHI": "%1.17e" % hi, "FS_HBINS": c.histBins,
                  "FS_HINVW": "%1.17e" % (c.histBins / float(hi - lo))})
    lines = [f"#define {k} {v}" for k, v in d.items()]
    return "\n".join(lines) + "\n", ft


def _user_section(c: OracleConfig, ft: str) -> str:
    args = ", ".join(f"FT x{i + 1}" for i in range(c.DOF))
    at = ", ".join(f"(p)[{i} * FS_N + (i)]" for i in range(c.DOF))
    out = [c.userCode or "", f"#define FS_ARGS_AT(p, i) {at}",
           f"static inline FT fs_pot({args}) {{ return ({c.potential}); }}"]

    def fn(name, exprs):
        body = " ".join(f"o[{i}] = ({e});" for i, e in enumerate(exprs))
        out.append(f"static inline void {name}({args}, FT *o) {{ {body} }}")

    if c.operators:
        fn("fs_ops", c.operators)
    if c.correlators:
        fn("fs_cors", c.correlators)
    if c.histograms and c.histBins > 0:
        fn("fs_hist", c.histograms)
    return "\n".join(out) + "\n"


def build(c: OracleConfig) -> str:
    with open(os.path.join(HERE, "pimc_oracle.c")) as f:
        tmpl = f.read()
    defines, ft = _defines(c)
    src = defines + tmpl.replace("/*@USER@*/", _user_section(c, ft))
    flags = ["-std=gnu11", "-O2", "-ffp-contract=off", "-fgnu89-inline", "-fopenmp",
             "-fPIC", "-shared", "-w"]
    if not c.enableDouble:
        flags.append("-fsingle-precision-constant")
    os.makedirs(BUILD, exist_ok=True)
    h = hashlib.sha1((src + " ".join(flags)).encode()).hexdigest()[:20]
    so = os.path.join(BUILD, f"oracle_{h}.so")
    if not os.path.exists(so):
        cpath = os.path.join(BUILD, f"oracle_{h}.c")
        with open(cpath, "w") as f:
            f.write(src)
        tmp = so + f".{os.getpid()}.tmp"
        r = subprocess.run(["gcc", *flags, "-I", HERE, cpath, "-o", tmp, "-lm"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr[-4000:])
        os.replace(tmp, so)
    return so


class _Args(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("paths", "accepts", "seeds", "walker_seeds", "ranlux_tab", "group_tab",
                 "op_means", "cor_means", "bins", "hist")] + \
               [("walker_begin", ctypes.c_int), ("walker_end", ctypes.c_int),
                ("omp_threads", ctypes.c_int), ("opnorm", ctypes.c_double),
                ("step_base", ctypes.c_ulonglong)]


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class OracleSampler:
    """Reference-semantics sampler on the CPU with numpy buffers in the reference layout."""
    cfg: OracleConfig
    omp_threads: int = 0
    lib: object = field(init=False, repr=False)

    def __post_init__(self):
        c = self.cfg
        self.lib = ctypes.CDLL(build(c))
        self.lib.fso_run.argtypes = [ctypes.POINTER(_Args)]
        self.lib.fso_run.restype = ctypes.c_int
        self.lib.fso_ranlux_init_rows.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        ft = np.float64 if c.enableDouble else np.float32
        W, T, nT = c.nbrOfWalkers, c.tpw, c.n_threads
        self.paths = np.zeros((W, c.N * c.DOF), ft)
        self.accepts = np.zeros(nT, np.uint32)
        self.seeds = np.zeros((nT + 1, 4), np.uint32)
        self.walker_seeds = np.zeros((W, 4), np.uint32)
        self.ranlux_tab = np.zeros((nT, 28), np.uint32)
        self.group_tab = np.zeros((nT if c.compat else W, 28), np.uint32)
        op_ft = {0: ft, 1: np.float64, 2: np.float32, 3: np.float64}[c.accum]
        nops = len(c.operators)
        self.op_means = np.zeros((nT, nops, 3) if c.accum == 3 else (nT * max(nops, 1),), op_ft)
        cor_ft = ft if c.accum == 0 else (COR_STUDY_DTYPE if c.accum == 3 else np.float64)
        self.cor_means = np.zeros((W, max(len(c.correlators), 1), c.N // 2), cor_ft)
        self.bins = np.zeros(c.binResolutionPerDOF ** c.DOF if c.enableBins else 1, np.uint32)
        self.hist = np.zeros(max(c.histBins, 1), np.uint64)
        self.launches = 0

    def init_ranlux_rows(self, table: np.ndarray, xs):
        xs = np.ascontiguousarray(np.asarray(xs, dtype=np.uint64))
        assert table.shape[0] == xs.shape[0]
        self.lib.fso_ranlux_init_rows(table.ctypes.data, int(xs.shape[0]), xs.ctypes.data)

    def run(self, walker_begin=0, walker_end=None):
        c = self.cfg
        a = _Args()
        for name in ("paths", "accepts", "seeds", "walker_seeds", "ranlux_tab", "group_tab",
                     "op_means", "cor_means", "bins", "hist"):
            arr = getattr(self, name)
            assert arr.flags["C_CONTIGUOUS"]
            setattr(a, name, _ptr(arr))
        a.walker_begin = walker_begin
        a.walker_end = c.nbrOfWalkers if walker_end is None else walker_end
        a.omp_threads = self.omp_threads or os.cpu_count() or 1
        a.opnorm = c.opnorm
        a.step_base = self.launches * c.operatorRuns * c.metroStepsPerOperatorRun
        rc = self.lib.fso_run(ctypes.byref(a))
        if rc != 0:
            raise RuntimeError(f"oracle run failed ({rc})")
        self.launches += 1


# ---- stand-alone RNG streams (no plugin needed) -------------------------------------
_RNG_C = r"""
#include "rng_oracle.h"
#include <string.h>
void fso_ranlux_stream(uint64_t x, int nskip, float *out, int n_calls, uint32_t *state_out)
{
    fso_ranlux_t st;
    fso_ranlux_init(&st, x);
    for (int i = 0; i < n_calls; i++) fso_ranlux32(&st, nskip, out + 4 * i);
    memcpy(state_out, &st, 112);
}
void fso_ranlux_stream64(uint64_t x, int nskip, double *out, int n_calls)
{
    fso_ranlux_t st;
    fso_ranlux_init(&st, x);
    for (int i = 0; i < n_calls; i++) fso_ranlux64(&st, nskip, out + 4 * i);
}
void fso_xorshift_stream(uint32_t *s, uint32_t *out, int n)
{
    for (int i = 0; i < n; i++) out[i] = fso_xorshift(s);
}
"""


def rng_lib():
    os.makedirs(BUILD, exist_ok=True)
    with open(os.path.join(HERE, "rng_oracle.h")) as f:
        h = hashlib.sha1((f.read() + _RNG_C).encode()).hexdigest()[:16]
    so = os.path.join(BUILD, f"rng_{h}.so")
    if not os.path.exists(so):
        cpath = os.path.join(BUILD, f"rng_{h}.c")
        with open(cpath, "w") as f:
            f.write(_RNG_C)
        tmp = so + f".{os.getpid()}.tmp"
        r = subprocess.run(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off",
                            "-fsingle-precision-constant", "-fPIC", "-shared", "-I", HERE,
                            cpath, "-o", tmp], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
        os.replace(tmp, so)
    lib = ctypes.CDLL(so)
    lib.fso_ranlux_stream.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_void_p]
    lib.fso_ranlux_stream64.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    lib.fso_xorshift_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    return lib


def ranlux_stream(x: int, lux_in_kernel: int, n_calls: int, double=False):
    lib = rng_lib()
    if double:
        out = np.zeros(4 * n_calls, np.float64)
        lib.fso_ranlux_stream64(x, nskip_for(lux_in_kernel), out.ctypes.data, n_calls)
        return out, None
    out = np.zeros(4 * n_calls, np.float32)
    st = np.zeros(28, np.uint32)
    lib.fso_ranlux_stream(x, nskip_for(lux_in_kernel), out.ctypes.data, n_calls, st.ctypes.data)
    return out, st


def xorshift_stream(state4, n: int):
    s = np.array(state4, dtype=np.uint32).copy()
    out = np.zeros(n, np.uint32)
    rng_lib().fso_xorshift_stream(s.ctypes.data, out.ctypes.data, n)
    return out, s
