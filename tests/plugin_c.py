"""FP64 evaluation of plugin C expressions on the CPU with gcc (test infrastructure).

A plugin's userCode and expression strings are compiled as C with FLOAT_TYPE double, the
CUDA built-in rsqrt written out, and evaluated row by row at given coordinates."""
import ctypes
import hashlib
import os
import subprocess
import tempfile

import numpy as np

_BUILD = os.path.join(tempfile.gettempdir(), "fs_plugin_c")


def eval_exprs(user_code, exprs, dof, x):
    """values [m, len(exprs)] of the expressions at coordinates x [m, dof]"""
    decl = " ".join(f"double x{k + 1} = x[{k}];" for k in range(dof))
    fns = "".join(f"static double f{i}(const double *x) {{ {decl} return {e}; }}\n" for i, e in enumerate(exprs))
    calls = " ".join(f"out[(size_t)r * {len(exprs)} + {i}] = f{i}(x + (size_t)r * {dof});" for i in range(len(exprs)))
    src = ("#include <math.h>\n#include <stddef.h>\n#define FLOAT_TYPE double\n"
           "static inline double rsqrt(double v) { return 1.0 / sqrt(v); }\n" + user_code + "\n" + fns +
           "void plugin_eval(const double *x, int m, double *out)\n"
           "{ int r; for (r = 0; r < m; r++) { " + calls + " } }\n")
    os.makedirs(_BUILD, exist_ok=True)
    h = hashlib.sha1(src.encode()).hexdigest()[:16]
    so = os.path.join(_BUILD, f"plugin_{h}.so")
    if not os.path.exists(so):
        c = os.path.join(_BUILD, f"plugin_{h}.c")
        with open(c, "w") as f:
            f.write(src)
        tmp = f"{so}.{os.getpid()}.tmp"
        r = subprocess.run(["gcc", "-std=gnu11", "-O1", "-ffp-contract=off", "-fgnu89-inline", "-fPIC", "-shared",
                            "-w", c, "-o", tmp, "-lm"], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(r.stderr[-3000:])
        os.replace(tmp, so)
    lib = ctypes.CDLL(so)
    lib.plugin_eval.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.shape[0], len(exprs)))
    lib.plugin_eval(x.ctypes.data, x.shape[0], out.ctypes.data)
    return out
