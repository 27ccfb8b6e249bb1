"""The reference's own sweep timed on the host cores -- TEST INFRASTRUCTURE ONLY.

Only bench.py's reference arm and cpu_baseline leg, and tests/, use this module; the
product never does.

prepare(name, system, ka) -- where the reference tree is present: runs the reference's
  kernel.py (through oracle/build_ref.py's stub pyopencl) for a sample of a benchmarked
  workload and writes to oracle/_ref/ (git-ignored) one self-contained C file -- the
  kernel text kernel.py generates (FeynSimul/GPUsrc/kernel.c after its substitution,
  kernel.py:215-348) with the vendored RANLUXCL header (examples/pyopencl-ranluxcl.cl)
  inlined where kernel.c:90 includes it, oracle/cl_shim.h's OpenCL-on-C definitions and a
  work-group launcher -- plus a manifest of the NDRange and buffers and the seed tables
  kernel.py drew (kernel.py:396-426).
rate(name, seconds, threads) -- wherever those files are, the reference tree not needed:
  compiles the C file with gcc for this machine with the reference's build options
  (kernel.py:371-376: fast relaxed math and single-precision constants, here -O3
  -ffast-math -fsingle-precision-constant), seeds the RANLUX tables with the reference's
  own init kernels, and runs the metropolis kernel the way a CPU OpenCL implementation runs
  work-groups: the work-items of one group as fibers (ucontext) on one OS thread, handing
  over at every barrier(), the groups spread over the host threads.

In the xorshift mode the reference's work-items read a shared offset-seed row at their start
and write it at their end (kernel.c:568-572, :832-835), so work-groups that run one after
another see each other's writes, as they may on an OpenCL device; only RANLUX samples are
timed, and the tests compare xorshift runs of one work-group.

Two textual changes are applied to the generated text, never to the reference's files: the
OpenCL swizzle of build_ref.SWIZZLE, and the parallel-path mode's __local path array
(kernel.c:588-589), declared a thread-local static so that the fibers of a group, which
share an OS thread, share it as a work-group shares local memory.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import platform
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, "_ref")

LOCAL_DECL = "PATH_TYPE_KEYWORD FLOAT_TYPE workGroupPath["
LOCAL_DECL_C = "static _Thread_local FLOAT_TYPE workGroupPath["
RANLUX_INCLUDE = "#include <pyopencl-ranluxcl.cl>"

FAST_FLAGS = ["-std=gnu11", "-O3", "-ffast-math", "-fsingle-precision-constant", "-fgnu89-inline",
              "-fPIC", "-shared", "-w"]
# the parity build's flags (IEEE, no contraction): used by the tests that compare the fiber
# launcher with oracle/build_ref.py's one-thread-per-work-item launcher
EXACT_FLAGS = ["-std=gnu11", "-O2", "-fsingle-precision-constant", "-ffp-contract=off",
               "-fgnu89-inline", "-fPIC", "-shared", "-w"]

# Work-group launcher: fibers on the host threads.  Each fiber runs one work-item from the
# kernel's entry to its end; barrier() (cl_shim.h's hook) swaps back to the scheduler, which
# resumes the group's fibers in turn, so every work-item of the group reaches barrier k
# before any passes it.
_FIBERS = r"""
#include <stdlib.h>
#include <ucontext.h>
_Thread_local clsh_item_t clsh_item;
pthread_barrier_t *clsh_barrier;
#define CLSH_STACK (256 * 1024)
typedef struct { ucontext_t ctx; clsh_item_t item; int done; } clsh_fiber_t;
static _Thread_local ucontext_t clsh_sched;
static _Thread_local clsh_fiber_t *clsh_cur;
static _Thread_local void **clsh_args;
static _Thread_local int clsh_which;
static void clsh_yield(void) { swapcontext(&clsh_cur->ctx, &clsh_sched); }
static void clsh_entry(void)
{
    void **a = clsh_args;
    (void)a;
    switch (clsh_which) {
    case 0: metropolis(%(METRO_ARGS)s); break;
%(RANLUX_CASES)s
    }
    clsh_cur->done = 1;
}
typedef struct { int which; void **a; size_t g0, g1, l0, l1, next; int err; } clsh_grid_t;
static void *clsh_worker(void *p)
{
    clsh_grid_t *G = (clsh_grid_t *)p;
    const size_t nl = G->l0 * G->l1, ng0 = G->g0 / G->l0, ng = ng0 * (G->g1 / G->l1);
    clsh_fiber_t *f = (clsh_fiber_t *)calloc(nl, sizeof(clsh_fiber_t));
    char *stacks = (char *)malloc(nl * (size_t)CLSH_STACK);
    if (!f || !stacks) { G->err = 1; free(f); free(stacks); return 0; }
    clsh_args = G->a;
    clsh_which = G->which;
    clsh_barrier_hook = clsh_yield;
    for (;;) {
        const size_t grp = __atomic_fetch_add(&G->next, (size_t)1, __ATOMIC_RELAXED);
        if (grp >= ng) break;
        const size_t gx = grp %% ng0, gy = grp / ng0;
        size_t i;
        for (i = 0; i < nl; i++) {
            const size_t lx = i %% G->l0, ly = i / G->l0;
            clsh_item_t it = {{gx * G->l0 + lx, gy * G->l1 + ly, 0}, {lx, ly, 0}, {gx, gy, 0},
                              {G->g0, G->g1, 1}, {G->l0, G->l1, 1}};
            f[i].item = it;
            f[i].done = 0;
            getcontext(&f[i].ctx);
            f[i].ctx.uc_stack.ss_sp = stacks + i * (size_t)CLSH_STACK;
            f[i].ctx.uc_stack.ss_size = CLSH_STACK;
            f[i].ctx.uc_link = &clsh_sched;
            makecontext(&f[i].ctx, clsh_entry, 0);
        }
        int live = 1;
        while (live) {
            live = 0;
            for (i = 0; i < nl; i++) {
                if (f[i].done) continue;
                clsh_cur = &f[i];
                clsh_item = f[i].item;
                swapcontext(&clsh_sched, &f[i].ctx);
                if (!f[i].done) live = 1;
            }
        }
    }
    clsh_barrier_hook = 0;
    free(stacks);
    free(f);
    return 0;
}
int clsh_launch_groups(int which, void **a, size_t g0, size_t g1, size_t l0, size_t l1, int threads)
{
    clsh_grid_t G = {which, a, g0, g1, l0, l1, 0, 0};
    pthread_t th[256];
    int t, n = threads < 1 ? 1 : (threads > 256 ? 256 : threads);
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, 1 << 20);
    for (t = 0; t < n; t++)
        if (pthread_create(&th[t], &attr, clsh_worker, &G) != 0) { n = t; G.err = 1; break; }
    for (t = 0; t < n; t++) pthread_join(th[t], 0);
    pthread_attr_destroy(&attr);
    return G.err ? -1 : 0;
}
"""


def _manifest_path(name):
    return os.path.join(REF_BUILD, f"timing_{name}.json")


def prepare(name: str, system, ka: dict, np_seed: int = 0) -> str:
    """Write oracle/_ref/timing_<name>.{c,json,npz} for a sample of a workload (needs the
    reference tree).  Returns the manifest path."""
    from oracle import build_ref
    cap = build_ref.capture(ka, system, np_seed)
    k = cap["kernel"]
    if cap["local_size"] is None:
        g, l = (cap["global_size"][0], 1), (1, 1)   # walker mode: local size 1, as build_ref
    else:
        g, l = cap["global_size"], cap["local_size"]
    bufs, args, ranlux_cases = build_ref.kernel_buffers(k)
    src = cap["source"].replace(build_ref.SWIZZLE, build_ref.SWIZZLE_C)
    if k._enableParallelizePath and not k._enableGlobalPath:
        assert src.count(LOCAL_DECL) == 1
        src = src.replace(LOCAL_DECL, LOCAL_DECL_C)
    if k._enableRanlux:
        with open(os.path.join(build_ref.REFERENCE_ROOT, "examples", "pyopencl-ranluxcl.cl")) as f:
            ranlux = f.read()
        assert src.count(RANLUX_INCLUDE) == 1
        src = src.replace(RANLUX_INCLUDE, ranlux)
    with open(os.path.join(HERE, "cl_shim.h")) as f:
        shim = f.read()
    launcher = _FIBERS % {"METRO_ARGS": ", ".join(args), "RANLUX_CASES": ranlux_cases}
    c_text = shim + "\n" + src + "\n" + launcher
    os.makedirs(REF_BUILD, exist_ok=True)
    c_name = f"timing_{name}.c"
    with open(os.path.join(REF_BUILD, c_name), "w") as f:
        f.write(c_text)
    arrays = {f"buf{i}": np.ascontiguousarray(b.arr) for i, b in enumerate(bufs)}
    if k._enableRanlux:
        arrays["seeds"] = np.ascontiguousarray(k._seeds.arr)
        arrays["group_seeds"] = np.ascontiguousarray(k._groupSeeds.arr)
    np.savez(os.path.join(REF_BUILD, f"timing_{name}.npz"), **arrays)
    seg = 2 ** int(ka["S"])
    man = {"c": c_name, "sha1": hashlib.sha1(c_text.encode()).hexdigest(),
           "npz": f"timing_{name}.npz", "global": list(g), "local": list(l),
           "n_buffers": len(bufs), "ranlux": bool(k._enableRanlux), "double": bool(k._enableDouble),
           "walkers": int(ka["nbrOfWalkers"]), "N": int(ka["N"]), "S": int(ka["S"]), "DOF": int(system.DOF),
           "operatorRuns": int(ka["operatorRuns"]), "metroStepsPerOperatorRun": int(ka["metroStepsPerOperatorRun"]),
           "beta": float(ka["beta"]), "enableRanlux": bool(ka.get("enableRanlux")),
           "luxuaryFactor": ka.get("luxuaryFactor"),
           "sweeps_per_launch": int(ka["operatorRuns"]) * int(ka["metroStepsPerOperatorRun"]),
           "node_updates_per_launch": int(ka["nbrOfWalkers"]) * (int(ka["N"]) // seg) * (seg - 1)
           * int(ka["operatorRuns"]) * int(ka["metroStepsPerOperatorRun"])}
    path = _manifest_path(name)
    with open(path, "w") as f:
        json.dump(man, f, indent=1)
    return path


def manifest(name: str) -> dict:
    with open(_manifest_path(name)) as f:
        return json.load(f)


def matches(name: str, ka: dict) -> bool:
    """Whether the prepared sample is of the workload ka describes (all but the walker count)."""
    man = manifest(name)
    return (man["N"] == int(ka["N"]) and man["S"] == int(ka["S"])
            and man["operatorRuns"] == int(ka["operatorRuns"])
            and man["metroStepsPerOperatorRun"] == int(ka["metroStepsPerOperatorRun"])
            and abs(man["beta"] - float(ka["beta"])) <= 1e-12 * abs(float(ka["beta"]))
            and man["enableRanlux"] == bool(ka.get("enableRanlux"))
            and (not man["enableRanlux"] or man["luxuaryFactor"] == ka.get("luxuaryFactor")))


def available(name: str) -> bool:
    p = _manifest_path(name)
    if not os.path.isfile(p):
        return False
    with open(p) as f:
        man = json.load(f)
    return all(os.path.isfile(os.path.join(REF_BUILD, man[k])) for k in ("c", "npz"))


class FiberKernel:
    """The prepared reference kernel, compiled for this machine, on its own buffers."""

    def __init__(self, name: str, fast: bool = True):
        with open(_manifest_path(name)) as f:
            self.man = man = json.load(f)
        src = os.path.join(REF_BUILD, man["c"])
        with open(src) as f:
            c_text = f.read()
        if hashlib.sha1(c_text.encode()).hexdigest() != man["sha1"]:
            raise RuntimeError(f"{src} does not match its manifest")
        flags = list(FAST_FLAGS if fast else EXACT_FLAGS)
        if man["double"]:
            flags.remove("-fsingle-precision-constant")
        tag = hashlib.sha1((c_text + " ".join(flags)).encode()).hexdigest()[:16]
        so = os.path.join(REF_BUILD, f"timing_{name}_{platform.machine()}_{tag}.so")
        if not os.path.exists(so):
            tmp = f"{so}.{os.getpid()}.tmp"     # concurrent builds each write their own file
            r = subprocess.run(["gcc", *flags, src, "-o", tmp, "-lpthread", "-lm"],
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("reference timing build failed:\n" + r.stderr[-3000:])
            os.replace(tmp, so)
        self.lib = ctypes.CDLL(so)
        self.lib.clsh_launch_groups.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                                ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
        self.lib.clsh_launch_groups.restype = ctypes.c_int
        z = np.load(os.path.join(REF_BUILD, man["npz"]))
        self.bufs = [np.array(z[f"buf{i}"]) for i in range(man["n_buffers"])]
        self.seeds = np.array(z["seeds"]) if man["ranlux"] else None
        self.group_seeds = np.array(z["group_seeds"]) if man["ranlux"] else None

    def _launch(self, which, arrays, threads):
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        g, l = self.man["global"], self.man["local"]
        if self.lib.clsh_launch_groups(which, ptrs, g[0], g[1], l[0], l[1], int(threads)) != 0:
            raise RuntimeError("reference launch failed")

    def init_ranlux(self, threads):
        if self.man["ranlux"]:
            self._launch(1, [self.seeds, self.bufs[-2]], threads)
            self._launch(2, [self.group_seeds, self.bufs[-1]], threads)

    def set_paths(self, paths):
        p = self.bufs[0]
        p[...] = np.asarray(paths, dtype=p.dtype).reshape(p.shape)

    def run(self, threads):
        self._launch(0, self.bufs, threads)


def rate(name: str, paths, seconds: float = 10.0, threads: int = 1) -> dict:
    """Node updates/s of the prepared reference kernel on `threads` host threads: launches
    repeated until `seconds` have passed (at least one timed launch after one untimed)."""
    k = FiberKernel(name)
    k.init_ranlux(threads)
    k.set_paths(paths)
    k.run(threads)                      # untimed: first touch of the buffers
    launches, t0 = 0, time.perf_counter()
    while True:
        k.run(threads)
        launches += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    man = k.man
    nodes = launches * man["node_updates_per_launch"]
    return {"value": nodes / dt, "seconds": dt, "launches": launches, "node_updates": nodes,
            "walkers": man["walkers"], "sweeps": launches * man["sweeps_per_launch"]}


def prepare_bench_samples():
    """The sample bench.py's reference arm times: the He3 workload with 64 walkers and its
    measurement cadence (the reference has no pair-distance histogram).  The harmonic
    oscillator is not prepared: its correlator takes a work-group barrier per lag and slice
    (kernel.c:792), so fibers would time context switches rather than the reference."""
    import bench
    sysm, ka, _extra, _wl = bench.he3_setup(walkers=64)
    return {"he3": prepare("he3", sysm, ka)}


def _bench_paths(name):
    """The starting walkers bench.py gives the oracle's sample of the same workload."""
    import bench
    man = manifest(name)
    setup = {"he3": bench.he3_setup}[name]
    sysm, ka, _extra, _wl = setup(walkers=man["walkers"])
    return bench.initial_paths(sysm, ka, 7)


if __name__ == "__main__":
    # python -m oracle.ref_timing rate NAME SECONDS THREADS  (run from the repository root):
    # bench.py times the reference in a process of its own
    import sys
    _, cmd, name, seconds, threads = sys.argv
    assert cmd == "rate"
    print(json.dumps(rate(name, _bench_paths(name), seconds=float(seconds), threads=int(threads))))
