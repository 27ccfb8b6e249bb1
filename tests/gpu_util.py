"""Helpers shared by the GPU tests: build the engine, make PIMCKernels for golden cases."""
import types

import numpy as np
import pytest

from golden_cases import HO


def have_gpu():
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so.13")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def require_gpu():
    if not have_gpu():
        pytest.fail("no CUDA device visible: -m gpu tests need a GB300")


def engine():
    from feynsimul_gb300 import build
    build.build()
    from feynsimul_gb300 import kernel, kernel_args
    return kernel, kernel_args


def ho_system():
    return types.SimpleNamespace(**HO)


def kernel_for_case(ka_dict, compat=True, accumulation="fp32", fast=False, **extra):
    kernel, kernel_args = engine()
    d = dict(ka_dict)
    ka = kernel_args.KernelArgs(system=ho_system(), compat=compat, accumulation=accumulation,
                                fastMath=fast, seed=1, **extra, **{k: v for k, v in d.items()})
    return kernel.PIMCKernel(ka)


def masked(t):
    t = np.array(t).reshape(-1, 28).copy()
    t[:, 25] = 0
    return t
