"""Ragged batches: many independent He-4 cluster systems in one persistent launch.

No counterpart in the reference (one system per OpenCL program there).  The device side
is csrc/fs_batch.cuh (+ fs_batch_api.cu): every system keeps its own walkers, slice count
N, bisection level S, beta and walker count; systems with the same particle count share
one compiled plugin type; CTAs take tiles of walkers from a work counter, largest first;
the launch can be replayed from a CUDA graph.

The autotuner picks the CTA size and the segment width (threads per walker, i.e. S for
each N) by timing candidates on the actual batch, and caches the choice in a JSON file
keyed by the batch's signature.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time

import numpy as np

from . import _lib
from ._lib import FsBatchSystem, check, lib, strings


def ragged_workload(seed=0, n_systems=64, n_range=(3, 10), N_choices=(128, 256, 512, 1024),
                    T_range=(0.5, 2.0), walker_range=(1024, 8192)):
    """The seeded synthetic batch: particle counts U{3..10}, N in {128..1024}, T U(0.5, 2) K,
    walkers U{1024..8192} (rounded to a multiple of 32)."""
    rng = np.random.RandomState(seed)
    out = []
    for _ in range(n_systems):
        n = int(rng.randint(n_range[0], n_range[1] + 1))
        N = int(rng.choice(N_choices))
        T = float(rng.uniform(*T_range))
        W = int(rng.randint(walker_range[0], walker_range[1] + 1)) // 32 * 32
        out.append({"n": n, "N": N, "T": T, "walkers": W})
    return out


def choose_S(N, tpw_target, block, dof=None, smem_budget=200 * 1024):
    """Bisection level of one system: N / 2^S = tpw_target segment threads per walker, except
    where a walker's path fills most of a tile's shared memory (large clusters): then the
    walker gets up to the whole CTA (segments of at least 4 slices), so the tile does not
    leave warps idle at its barriers.  With segments of at least 8 slices, five of the
    standard workload's system types left 64-256 of a 512-thread CTA idle: 5.76e9 against
    6.44e9 node updates/s with 4."""
    S = int(np.log2(N)) - int(np.log2(tpw_target))
    S = max(1, min(S, 10, int(np.log2(N))))
    if dof is not None:
        walker_bytes = dof * (N + N // 8) * 4 + 512
        wpb_max = max(1, smem_budget // walker_bytes)
        if wpb_max * (N >> S) < block and N >= 8:
            tpw = 1 << int(np.log2(max(1, block // wpb_max)))
            tpw = min(tpw, N // 4)
            S = min(S, max(1, int(np.log2(N // tpw))))
    while (N >> S) > block:
        S += 1
    return S


class BatchSampler:
    """One persistent launch over all systems of a workload (list of dicts with n, N, T,
    walkers)."""

    def __init__(self, workload, op_runs=1, msteps=4, block_threads=256, tpw_target=16, seed=0, noise=0.0,
                 ranlux=None):
        """ranlux: None for xorshift streams, or a luxuaryFactor (the kernel uses +1, as
        KernelArgs.luxuaryFactor) for RANLUX tables, seeded per system like the sweep's fixed
        mode: thread row r from (s << 32) + r, walker row w from ((s ^ 2^31) << 32) + w, s a
        31-bit seed drawn per system."""
        from .physical_systems.lm2m2 import Lm2m2Cluster
        self.workload = workload
        ns = sorted({w["n"] for w in workload})
        self.type_of = {n: k for k, n in enumerate(ns)}
        clusters = {n: Lm2m2Cluster(n, 1.0) for n in ns}
        self.clusters = clusters
        self.op_runs, self.msteps, self.block = op_runs, msteps, block_threads
        self.systems = []
        for w in workload:
            c = clusters[w["n"]]
            S = choose_S(w["N"], tpw_target, block_threads, dof=c.DOF)
            self.systems.append(FsBatchSystem(type=self.type_of[w["n"]], n_walkers=w["walkers"], n_slices=w["N"],
                                              bisection_level=S, beta=1.0 / w["T"], walkers_per_tile=0))
        arr = (FsBatchSystem * len(self.systems))(*self.systems)
        dofs = (ctypes.c_int32 * len(ns))(*[clusters[n].DOF for n in ns])
        pots, _ = strings([clusters[n].potential for n in ns])
        ucs, _ = strings([clusters[n].userCode for n in ns])
        ops, _ = strings([clusters[n].energyOp for n in ns])
        h = ctypes.c_void_p()
        self.ranlux = ranlux
        check(lib().fs_batch_create(len(ns), dofs, pots, ucs, ops, 1, len(self.systems), arr, op_runs, msteps,
                                    block_threads, -1 if ranlux is None else int(ranlux), ctypes.byref(h)))
        self._h = h
        L = lib()
        nu, sm, rg, ni, gr = (ctypes.c_int64() for _ in range(5))
        wpt = (ctypes.c_int64 * len(self.systems))()
        check(L.fs_batch_query(h, ctypes.byref(nu), ctypes.byref(sm), ctypes.byref(rg), ctypes.byref(ni),
                               ctypes.byref(gr), wpt, len(self.systems)))
        self.node_updates_per_launch = nu.value
        self.smem, self.registers, self.n_items, self.grid = sm.value, rg.value, ni.value, gr.value
        self.walkers_per_tile = list(wpt)
        rng = np.random.RandomState(seed)
        for i, (w, s) in enumerate(zip(workload, self.systems)):
            c = clusters[w["n"]]
            paths = c.initial_paths(w["walkers"], w["N"], rng, noise=noise).astype(np.float32)
            check(L.fs_batch_set_paths(h, i, paths.ctypes.data, paths.size))
            tpw = w["N"] >> s.bisection_level
            ts = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"] * tpw, 4)).astype(np.uint32)
            ws = rng.randint(0, 2 ** 31 - 1, size=(w["walkers"], 4)).astype(np.uint32)
            check(L.fs_batch_set_seeds(h, i, ts.ctypes.data, ts.shape[0], ws.ctypes.data, ws.shape[0]))
            if ranlux is not None:
                base = int(rng.randint(0, 2 ** 31 - 1))
                xt = (np.uint64(base) << np.uint64(32)) + np.arange(ts.shape[0], dtype=np.uint64)
                xw = (np.uint64(base ^ 0x80000000) << np.uint64(32)) + np.arange(ws.shape[0], dtype=np.uint64)
                check(L.fs_batch_init_ranlux(h, i, xt.ctypes.data, xt.size, xw.ctypes.data, xw.size))

    def ranlux_tables(self, i):
        """System i's RANLUX tables (thread rows [threads][28], walker rows [walkers][28],
        uint32, the reference's layout)."""
        s = self.systems[i]
        nt = s.n_walkers * (s.n_slices >> s.bisection_level)
        t = np.empty((nt, 28), np.uint32)
        g = np.empty((s.n_walkers, 28), np.uint32)
        check(lib().fs_batch_get_ranlux_tables(self._h, i, t.ctypes.data, nt, g.ctypes.data, s.n_walkers))
        return t, g

    def set_state(self, i, paths, thread_seeds, walker_seeds):
        """Replace system i's paths [walkers, DOF*N] and xorshift rows ([walkers*tpw][4] per
        thread, thread = walker*tpw + t; [walkers][4] per walker)."""
        L = lib()
        p = np.ascontiguousarray(paths, np.float32)
        ts = np.ascontiguousarray(thread_seeds, np.uint32)
        ws = np.ascontiguousarray(walker_seeds, np.uint32)
        check(L.fs_batch_set_paths(self._h, i, p.ctypes.data, p.size))
        check(L.fs_batch_set_seeds(self._h, i, ts.ctypes.data, ts.shape[0], ws.ctypes.data, ws.shape[0]))

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().fs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, launches=1, graph=True):
        check(lib().fs_batch_run(self._h, int(launches), int(bool(graph))))
        check(lib().fs_batch_sync(self._h))
        t = ctypes.c_double()
        check(lib().fs_batch_get_run_time(self._h, ctypes.byref(t)))
        return t.value

    def energy_sums(self, i):
        W = self.workload[i]["walkers"]
        out = np.empty(W, np.float64)
        check(lib().fs_batch_get_op_sums(self._h, i, out.ctypes.data, W))
        return out

    def paths(self, i):
        w = self.workload[i]
        out = np.empty(w["walkers"] * self.clusters[w["n"]].DOF * w["N"], np.float32)
        check(lib().fs_batch_get_paths(self._h, i, out.ctypes.data, out.size))
        return out.reshape(w["walkers"], -1)

    def accepts(self, i):
        s = self.systems[i]
        n = s.n_walkers * (s.n_slices >> s.bisection_level)
        out = np.empty(n, np.uint32)
        check(lib().fs_batch_get_accepts(self._h, i, out.ctypes.data, n))
        return out


# bumped when the batch kernel or its launch-shape rules change, so cached tunings expire
_TUNING_VERSION = 4


def _signature(workload, op_runs, msteps):
    return hashlib.sha1(json.dumps([workload, op_runs, msteps, _TUNING_VERSION],
                                   sort_keys=True).encode()).hexdigest()[:16]


def autotune(workload, op_runs=1, msteps=4, candidates=None, cache_file=None, launches=2, log=None):
    """Time each (block_threads, threads-per-walker target) candidate on the batch and return
    the fastest as a dict; cached in cache_file (JSON) by the batch signature."""
    cache_file = cache_file or os.path.join(os.environ.get("FS_CACHE_DIR", os.path.expanduser(
        "~/.cache/feynsimul_gb300")), "batch_autotune.json")
    key = _signature(workload, op_runs, msteps)
    cache = {}
    if os.path.exists(cache_file):
        try:
            cache = json.load(open(cache_file))
        except ValueError:
            cache = {}
    if key in cache:
        return dict(cache[key], cached=True)
    shipped = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned", "batch_autotune.json")
    if os.path.exists(shipped):
        try:
            tuned = json.load(open(shipped))
        except ValueError:
            tuned = {}
        if key in tuned:
            return dict(tuned[key], cached=True, shipped=True)
    candidates = candidates or [(512, 32), (256, 32), (512, 16), (256, 16), (512, 64)]
    results = []
    for block, tpw in candidates:
        try:
            b = BatchSampler(workload, op_runs, msteps, block, tpw)
        except _lib.FsError as e:
            results.append({"block_threads": block, "tpw_target": tpw, "error": str(e)[:200]})
            continue
        b.run(1)
        t = b.run(launches) / launches
        r = {"block_threads": block, "tpw_target": tpw, "s_per_launch": t,
             "node_updates_per_s": b.node_updates_per_launch / t, "registers": b.registers, "smem": b.smem}
        if log:
            log(r)
        results.append(r)
        b.close()
    ok = [r for r in results if "error" not in r]
    best = max(ok, key=lambda r: r["node_updates_per_s"])
    best = dict(best, candidates=results)
    os.makedirs(os.path.dirname(cache_file), exist_ok=True)
    cache[key] = best
    tmp = cache_file + f".{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1)
    os.replace(tmp, cache_file)
    return dict(best, cached=False)
