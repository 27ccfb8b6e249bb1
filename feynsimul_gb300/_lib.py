"""ctypes binding of libfeynsimul_gb300.so (include/feynsimul.h).

The library is loaded from the package directory.  There is no fallback: when the shared
object is missing the import of a GPU entry point raises, naming the build command.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libfeynsimul_gb300.so")

FS_OK = 0
FS_ERR_CONFIG = -1
FS_ERR_COMPILE = -2
FS_ERR_OOM = -3
FS_ERR_LAUNCH = -4
FS_ERR_TIMEOUT = -5
FS_ERR_IO = -6
FS_ERR_CUDA = -7
FS_ERR_STATE = -8
FS_ERR_NUMERIC = -9

ACCUM_REF_FP32, ACCUM_FP64, ACCUM_KAHAN, ACCUM_STUDY = 0, 1, 2, 3

# Every symbol include/feynsimul.h declares (checked by tests/test_boundary.py).
EXPORTS = (
    "fs_create", "fs_destroy", "fs_compile_only", "fs_last_error", "fs_build_log", "fs_source",
    "fs_query", "fs_set_paths", "fs_get_paths", "fs_set_xorshift_seeds", "fs_get_xorshift_seeds",
    "fs_set_walker_seeds", "fs_get_walker_seeds", "fs_ranlux_init", "fs_ranlux_group_init",
    "fs_get_ranlux_tables", "fs_set_ranlux_tables", "fs_run", "fs_sync", "fs_sync_timeout",
    "fs_get_operators", "fs_get_correlator", "fs_get_accepts", "fs_get_bins", "fs_get_histogram",
    "fs_zero_accumulators", "fs_get_run_time", "fs_rng_ranlux_stream", "fs_rng_ranlux_stream64",
    "fs_rng_xorshift_stream", "fs_version", "fs_ranlux_init_noalloc", "fs_set_correlator",
    "fs_set_bins", "fs_set_histogram", "fs_mlp_sizes", "fs_mlp_train_step", "fs_mlp_adam",
    "fs_mlp_pack", "fs_mlp_infer", "fs_set_learned_proposal", "fs_batch_create", "fs_batch_destroy",
    "fs_batch_run", "fs_batch_sync", "fs_batch_get_run_time", "fs_batch_set_paths", "fs_batch_get_paths",
    "fs_batch_set_seeds", "fs_batch_init_ranlux", "fs_batch_get_ranlux_tables", "fs_batch_get_op_sums",
    "fs_batch_get_accepts", "fs_batch_query",
    "fs_reduce_correlator", "fs_set_paths_tiled", "fs_get_step_counter", "fs_set_step_counter",
    "fs_run_host", "fs_pin_host", "fs_unpin_host", "fs_get_walker_operators", "fs_get_last_chunks",
)

FS_MOVE_BISECTION, FS_MOVE_PATH_SHIFT, FS_MOVE_SINGLE_NODE = 1, 2, 4
FS_PARTIALS_FP32, FS_PARTIALS_EXACT = 0, 1


class FsConfig(ctypes.Structure):
    _fields_ = [
        ("dof", ctypes.c_int32), ("n_slices", ctypes.c_int32), ("bisection_level", ctypes.c_int32),
        ("beta", ctypes.c_double), ("n_walkers", ctypes.c_int32), ("walkers_per_group", ctypes.c_int32),
        ("operator_runs", ctypes.c_int32), ("metro_steps_per_operator_run", ctypes.c_int32),
        ("enable_parallelize_path", ctypes.c_int32), ("enable_ranlux", ctypes.c_int32),
        ("luxury_factor", ctypes.c_int32), ("ranlux_int_max", ctypes.c_uint64),
        ("enable_double", ctypes.c_int32), ("enable_bins", ctypes.c_int32),
        ("x_min", ctypes.c_double), ("x_max", ctypes.c_double),
        ("bin_resolution_per_dof", ctypes.c_int32),
        ("hist_lo", ctypes.c_double), ("hist_hi", ctypes.c_double), ("hist_bins", ctypes.c_int32),
        ("compat", ctypes.c_int32), ("accum", ctypes.c_int32), ("fast_math", ctypes.c_int32),
        ("walkers_per_block", ctypes.c_int32), ("min_blocks_per_sm", ctypes.c_int32),
        ("learned", ctypes.c_int32), ("global_path", ctypes.c_int32), ("potential_cache", ctypes.c_int32),
        ("moves", ctypes.c_int32), ("alpha", ctypes.c_double), ("ps_alpha", ctypes.c_double),
        ("partials", ctypes.c_int32),
    ]


class FsInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "n_threads", "threads_per_walker", "walkers_per_block", "block_threads", "grid_blocks",
        "smem_bytes", "registers", "device_bytes", "uniforms_per_move", "nodes_per_move", "potential_cache")]


class FsBatchSystem(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("n_walkers", ctypes.c_int32), ("n_slices", ctypes.c_int32),
                ("bisection_level", ctypes.c_int32), ("beta", ctypes.c_double),
                ("walkers_per_tile", ctypes.c_int32)]


class FsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None

_P = ctypes.c_void_p
_S = ctypes.c_size_t
_I = ctypes.c_int32
_STRS = ctypes.POINTER(ctypes.c_char_p)

_PROTOS = {
    "fs_create": ([ctypes.POINTER(FsConfig), ctypes.c_char_p, ctypes.c_char_p, _STRS, _I, _STRS, _I,
                   _STRS, _I, ctypes.POINTER(_P)], ctypes.c_int),
    "fs_compile_only": ([ctypes.POINTER(FsConfig), ctypes.c_char_p, ctypes.c_char_p, _STRS, _I, _STRS, _I,
                         _STRS, _I, ctypes.c_char_p, _S], ctypes.c_int),
    "fs_destroy": ([_P], ctypes.c_int),
    "fs_last_error": ([_P], ctypes.c_char_p),
    "fs_build_log": ([_P], ctypes.c_char_p),
    "fs_source": ([_P], ctypes.c_char_p),
    "fs_version": ([], ctypes.c_char_p),
    "fs_query": ([_P, ctypes.POINTER(FsInfo)], ctypes.c_int),
    "fs_set_paths": ([_P, _P, _S], ctypes.c_int),
    "fs_get_paths": ([_P, _P, _S], ctypes.c_int),
    "fs_set_xorshift_seeds": ([_P, _P, _S], ctypes.c_int),
    "fs_get_xorshift_seeds": ([_P, _P, _S], ctypes.c_int),
    "fs_set_walker_seeds": ([_P, _P, _S], ctypes.c_int),
    "fs_get_walker_seeds": ([_P, _P, _S], ctypes.c_int),
    "fs_ranlux_init": ([_P, _P, _S], ctypes.c_int),
    "fs_ranlux_group_init": ([_P, _P, _S], ctypes.c_int),
    "fs_get_ranlux_tables": ([_P, _P, _S, _P, _S], ctypes.c_int),
    "fs_set_ranlux_tables": ([_P, _P, _S, _P, _S], ctypes.c_int),
    "fs_run": ([_P, _I], ctypes.c_int),
    "fs_sync": ([_P], ctypes.c_int),
    "fs_sync_timeout": ([_P, ctypes.c_double], ctypes.c_int),
    "fs_get_operators": ([_P, _P, _S], ctypes.c_int),
    "fs_get_correlator": ([_P, _P, _S], ctypes.c_int),
    "fs_reduce_correlator": ([_P, ctypes.c_int64, ctypes.c_int64, _P, _P, _S], ctypes.c_int),
    "fs_set_paths_tiled": ([_P, _P, _S], ctypes.c_int),
    "fs_get_step_counter": ([_P, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "fs_run_host": ([_P, _P, _P, _I, _I], ctypes.c_int),
    "fs_get_walker_operators": ([_P, _P, _S], ctypes.c_int),
    "fs_get_last_chunks": ([_P, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "fs_pin_host": ([_P, _S], ctypes.c_int),
    "fs_unpin_host": ([_P], ctypes.c_int),
    "fs_set_step_counter": ([_P, ctypes.c_uint64], ctypes.c_int),
    "fs_get_accepts": ([_P, _P, _S], ctypes.c_int),
    "fs_get_bins": ([_P, _P, _S], ctypes.c_int),
    "fs_get_histogram": ([_P, _P, _S], ctypes.c_int),
    "fs_zero_accumulators": ([_P], ctypes.c_int),
    "fs_get_run_time": ([_P, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "fs_rng_ranlux_stream": ([_I, _P, _I, _I, _P, _P], ctypes.c_int),
    "fs_rng_ranlux_stream64": ([_I, _P, _I, _I, _P], ctypes.c_int),
    "fs_rng_xorshift_stream": ([_P, _I, _I, _P, _P], ctypes.c_int),
    "fs_ranlux_init_noalloc": ([_P, _P, _S, _P], ctypes.c_int),
    "fs_set_correlator": ([_P, _P, _S], ctypes.c_int),
    "fs_set_bins": ([_P, _P, _S], ctypes.c_int),
    "fs_set_histogram": ([_P, _P, _S], ctypes.c_int),
    "fs_mlp_sizes": ([_P, _P, _P, _P], ctypes.c_int),
    "fs_mlp_train_step": ([_P, _P, _P, _P, _P, _I, _I, ctypes.c_float, _P, _P], ctypes.c_int),
    "fs_mlp_adam": ([_P, _P, _P, _P, _P, _I, ctypes.c_float, _P], ctypes.c_int),
    "fs_mlp_pack": ([_P, _P, _P, _P, _P], ctypes.c_int),
    "fs_mlp_infer": ([_P, _P, _P, _P, _I, _P], ctypes.c_int),
    "fs_set_learned_proposal": ([_P, _P, _S, _P, _S, ctypes.c_double], ctypes.c_int),
    "fs_batch_create": ([_I, _P, _STRS, _STRS, _STRS, _I, _I, _P, _I, _I, _I, _I, ctypes.POINTER(_P)], ctypes.c_int),
    "fs_batch_init_ranlux": ([_P, _I, _P, _S, _P, _S], ctypes.c_int),
    "fs_batch_get_ranlux_tables": ([_P, _I, _P, _S, _P, _S], ctypes.c_int),
    "fs_batch_destroy": ([_P], ctypes.c_int),
    "fs_batch_run": ([_P, _I, _I], ctypes.c_int),
    "fs_batch_sync": ([_P], ctypes.c_int),
    "fs_batch_get_run_time": ([_P, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "fs_batch_set_paths": ([_P, _I, _P, _S], ctypes.c_int),
    "fs_batch_get_paths": ([_P, _I, _P, _S], ctypes.c_int),
    "fs_batch_set_seeds": ([_P, _I, _P, _S, _P, _S], ctypes.c_int),
    "fs_batch_get_op_sums": ([_P, _I, _P, _S], ctypes.c_int),
    "fs_batch_get_accepts": ([_P, _I, _P, _S], ctypes.c_int),
    "fs_batch_query": ([_P, _P, _P, _P, _P, _P, _P, _S], ctypes.c_int),
}


def lib():
    """Load the shared object (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m feynsimul_gb300.build` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (argt, rest) in _PROTOS.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = rest
        _lib = L
    return _lib


def strings(seq):
    seq = [s.encode() if isinstance(s, str) else s for s in seq]
    arr = (ctypes.c_char_p * max(1, len(seq)))(*seq)
    return arr, len(seq)


def check(rc, handle=None):
    if rc != FS_OK:
        msg = lib().fs_last_error(handle)
        raise FsError(rc, msg.decode(errors="replace") if msg else "")
    return rc
