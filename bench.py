"""Benchmark: path-node updates/s of the Metropolis-bisection sweep on GB300.

Workload (default ``--config he3``): three He-4 atoms with the LM2M2 pair potential,
T = 1 K (beta = 1/K), N = 256 slices, bisection level S = 4, 16384 walkers, RANLUX
(luxuaryFactor 2), FP32 paths, FP64 operator sums; operators: the virial energy and a
200-bin pair-distance histogram on 0-20 Angstrom.  Paths start as random equilateral
triangles of side U(3, 5) Angstrom plus N(0, 0.1 Angstrom) noise (seeded).

A step is one PIMCKernel.run(): operatorRuns x metroStepsPerOperatorRun sweeps of every
walker in one kernel launch.  A node update is one interior time slice (all DOF)
resampled by a bisection move, accepted or not: walkers x N/2^S segments x (2^S - 1)
per sweep.

value: node updates/s with the state resident in HBM (CUDA events around each launch,
L2 flushed between launches).  e2e: the same through the reference-facing API with host
buffers: each step copies the paths in from pinned host memory, runs, and reads the
operator means and the paths back.  cpu_baseline: the oracle's C restatement of the
reference sweep on the host cores (OpenMP) on a bounded sample of the same workload.

``--impl reference`` times the reference algorithm on the CPU instead (the oracle port,
every host thread): the reference's OpenCL kernels have no runnable OpenCL platform here.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


# ------------------------------------------------------------------ workloads
def he3_setup(walkers=16384, N=256, S=4, op_runs=5, msteps=10):
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    sysm = Lm2m2Cluster(3, 1.0)
    ka = dict(nbrOfWalkers=walkers, N=N, beta=float(sysm.beta), S=S, enableOperator=True,
              enableCorrelator=False, enableBisection=True, enablePathShift=False,
              enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
              enableParallelizePath=True, enableGlobalPath=False, enableGlobalOldPath=False,
              enableDouble=False, enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
              operators=(sysm.energyOp,), operatorRuns=op_runs, metroStepsPerOperatorRun=msteps)
    extra = dict(histograms=sysm.pairDistanceOps, histRange=(0.0, 20.0), histBins=200)
    workload = (f"He3 LM2M2 T=1K N={N} S={S} walkers={walkers} RANLUX lux2 fp32 paths, "
                f"fp64 sums, energy + 200-bin pair-distance histogram")
    return sysm, ka, extra, workload


def ho_setup(walkers=1024, N=128, S=3, op_runs=100, msteps=1):
    from feynsimul_gb300.physical_systems.harm_osc import HarmOsc
    sysm = HarmOsc()
    ka = dict(nbrOfWalkers=walkers, N=N, beta=10.0, S=S, enableOperator=True, enableCorrelator=True,
              enableBisection=True, enablePathShift=False, enableSingleNodeMove=False, enableBins=False,
              nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
              enableGlobalOldPath=False, enableDouble=False, enableRanlux=False,
              operators=(sysm.energyOp,), correlators=("x1",), operatorRuns=op_runs,
              metroStepsPerOperatorRun=msteps)
    return sysm, ka, {}, f"1D HO beta=10 N={N} S={S} walkers={walkers} xorshift, x^2 and <x(0)x(t)>"


def initial_paths(sysm, ka, seed):
    rng = np.random.RandomState(seed)
    if hasattr(sysm, "initial_paths"):
        return sysm.initial_paths(ka["nbrOfWalkers"], ka["N"], rng).astype(np.float32)
    return np.zeros((ka["nbrOfWalkers"], ka["N"] * sysm.DOF), np.float32)


def workload_overrides(args):
    o = {}
    if args.walkers:
        o["walkers"] = args.walkers
    if args.op_runs:
        o["op_runs"] = args.op_runs
    if args.msteps:
        o["msteps"] = args.msteps
    if args.S:
        o["S"] = args.S
    return o


def bench_config(workload, ka):
    """The workload keys of the JSON line, identical in both arms (the reference arm times a
    bounded sample of the same workload; its sample is described in its cpu_baseline)."""
    return {"workload": workload, "sweeps_per_step": ka["operatorRuns"] * ka["metroStepsPerOperatorRun"],
            "node_updates_per_step": node_updates_per_run(ka)}


def _json_safe(obj):
    if isinstance(obj, dict):
        return {k: _json_safe(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [_json_safe(v) for v in obj]
    if isinstance(obj, np.ndarray):
        return obj.tolist()
    if isinstance(obj, np.generic):
        return obj.item()
    return obj


def node_updates_per_run(ka):
    seg = 2 ** ka["S"]
    tpw = ka["N"] // seg
    return ka["nbrOfWalkers"] * tpw * (seg - 1) * ka["operatorRuns"] * ka["metroStepsPerOperatorRun"]


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        return self.summarize(self.lines)

    @staticmethod
    def summarize(lines):
        """Median SM clock, the maximum, and every throttle reason seen active in the
        sampled CSV lines (the query's column order)."""
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f)
    except OSError:
        return None


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_cpu_rate(sysm, ka, extra, seconds=10.0, walkers=None):
    """Node updates/s of the oracle's C restatement (the reference algorithm) on the host
    cores, on a bounded sample: a subset of walkers and fewer operator runs, sized to
    ~seconds, with the workload's measurement cadence (metroStepsPerOperatorRun sweeps per
    measurement of the operators, correlators and histograms)."""
    from oracle import oracle as orc
    cores = cpu_cores()
    W = walkers or max(cores * 4, 64)
    W = min(W, ka["nbrOfWalkers"])

    msteps = int(ka["metroStepsPerOperatorRun"])

    def make(runs):
        cfg = orc.OracleConfig(
            DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=W, N=ka["N"],
            beta=ka["beta"], S=ka["S"], operatorRuns=runs, metroStepsPerOperatorRun=msteps,
            nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableRanlux=ka["enableRanlux"],
            luxuaryFactor=ka.get("luxuaryFactor", 2), ranluxIntMax=ka.get("ranluxIntMax", 2 ** 32 - 1),
            operators=ka["operators"], correlators=ka.get("correlators", ()) or (), compat=False, accum=1,
            histograms=extra.get("histograms", ()), histRange=extra.get("histRange", (0.0, 1.0)),
            histBins=extra.get("histBins", 0))
        o = orc.OracleSampler(cfg, omp_threads=cores)
        o.paths[...] = initial_paths(sysm, dict(ka, nbrOfWalkers=W), 7)
        if ka["enableRanlux"]:
            o.init_ranlux_rows(o.ranlux_tab, (np.uint64(12345) << np.uint64(32)) + np.arange(o.ranlux_tab.shape[0], dtype=np.uint64))
            o.init_ranlux_rows(o.group_tab, (np.uint64(54321) << np.uint64(32)) + np.arange(o.group_tab.shape[0], dtype=np.uint64))
        else:
            rs = np.random.RandomState(1)
            o.seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.seeds.shape)
            o.walker_seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape)
        return o, cfg

    # calibrate on growing samples until one takes a tenth of the target, then scale
    runs = 4
    while True:
        o, cfg = make(runs)
        t0 = time.perf_counter()
        o.run()
        t1 = time.perf_counter() - t0
        if t1 >= 0.1 * seconds or runs >= 10 ** 6:
            break
        runs = int(min(10 ** 6, runs * max(2.0, 0.15 * seconds / max(t1, 1e-6))))
    runs = int(max(1, min(10 ** 6, runs * seconds / max(t1, 1e-6))))
    o, cfg = make(runs)
    t0 = time.perf_counter()
    o.run()
    dt = time.perf_counter() - t0
    seg = 2 ** ka["S"]
    sweeps = runs * msteps
    nodes = W * (ka["N"] // seg) * (seg - 1) * sweeps
    return {"value": nodes / dt, "unit": "node-updates/s", "cores": cores, "kind": "port", "seconds": dt,
            "sample": f"{W} walkers x {sweeps} sweeps of the same system, one measurement every {msteps} "
                      f"sweep(s) ({nodes} node updates, {dt:.1f} s), oracle C restatement, OpenMP over walkers"}


def reference_cpu_rate(config, sysm, ka, extra, seconds=10.0):
    """Node updates/s of the reference's own sweep on the host cores: its kernel.c and
    RANLUXCL as its kernel.py generates them for a 64-walker sample of the He3 workload,
    compiled with its fast-relaxed-math build and run as a CPU OpenCL implementation runs
    work-groups (oracle/ref_timing.py), where oracle/_ref holds that sample.  Otherwise, and
    for the harmonic oscillator, the oracle's C restatement: the reference's correlator takes
    a work-group barrier per lag and slice (kernel.c:792), which an execution of the
    work-items as fibers turns into context switches that no OpenCL compiler would make."""
    reason = "the reference sample is prepared for the He3 workload only"
    if config == "he3":
        try:
            from oracle import ref_timing
            if not ref_timing.available("he3"):
                reason = "oracle/_ref holds no prepared sample (the reference tree was absent at build time)"
            elif not ref_timing.matches("he3", ka):
                reason = "the prepared sample is of another configuration"
            else:
                # in a process of its own, so that nothing the host build does can touch this one
                cores = cpu_cores()
                man = ref_timing.manifest("he3")
                root = os.path.dirname(os.path.abspath(__file__))
                pr = subprocess.run([sys.executable, "-m", "oracle.ref_timing", "rate", "he3", str(seconds),
                                     str(cores)], cwd=root, capture_output=True, text=True,
                                    timeout=3 * seconds + 300)
                if pr.returncode != 0:
                    raise RuntimeError(f"exit {pr.returncode}: {pr.stderr.strip()[-300:]}")
                r = json.loads(pr.stdout.strip().splitlines()[-1])
                return {"value": r["value"], "unit": "node-updates/s", "cores": cores, "kind": "reference",
                        "seconds": r["seconds"],
                        "sample": f"{r['walkers']} walkers x {r['sweeps']} sweeps of the same system, one "
                                  f"measurement of the energy every {man['metroStepsPerOperatorRun']} sweeps (the "
                                  f"reference has no pair-distance histogram); the reference's kernel.c + "
                                  f"RANLUXCL generated by its kernel.py, gcc -O3 -ffast-math (its fast relaxed "
                                  f"math build), the work-items of a group as fibers, groups over {cores} host "
                                  f"threads"}
        except Exception as e:  # the restatement stands in; the reason is reported
            reason = f"{type(e).__name__}: {str(e)[:300]}"
    cb = oracle_cpu_rate(sysm, ka, extra, seconds=seconds)
    cb["reference_unavailable"] = reason
    return cb


# register budget the sweep kernel is compiled for, per workload (launch-shape sweep on GB300)
TUNED_MIN_BLOCKS = {"he3": 7, "ho": 0}
TUNED_WPB = {"he3": 4, "ho": 0}


# ------------------------------------------------------------------ roofline
# Algorithmic lane operations per node update (one interior slice, all DOF, resampled by a
# bisection move), counted from the algorithm, not from the executed code:
#   RNG    2*DOF uniforms (+ amortised accept / offset draws); RANLUX p = 24 + NSKIP steps of
#          subtract-with-borrow per 24 uniforms, 3 integer ops each, + 4 ops per output and
#          4 for the buffered hand-out; xorshift 6 ops per uniform + 2 to convert
#   BM     per DOF: log, sqrt, sin (1 op each, SFU) + 6 multiplies/adds for the midpoint
#   V      two potential evaluations per node (old and new path); LM2M2 trimer: 15 ops for
#          the positions, 3 pairs x (6 ops for r^2 + 35 for the pair potential) = 138;
#          harmonic oscillator: 3
# The peak is the issue roof of the SMs: 4 schedulers x 32 lanes x 152 SMs per clock, at
# the median SM clock sampled during the timed region (one lane op per lane per cycle).
POT_OPS = {"he3": 138.0, "ho": 3.0}
# lane operations per slice of one measurement: He3 the virial energy (3 pairs with the
# LM2M2 derivative) and the 200-bin histogram of the 3 pair distances; HO x^2
MEAS_OPS = {"he3": 3 * 60.0 + 3 * 12.0, "ho": 2.0}


def alg_ops_per_node(config, ka):
    """Algorithmic lane operations per node update: the move (random numbers, Box-Muller,
    two potential evaluations) plus the launch's measurements spread over its node updates
    (operators and histogram per slice, and for a correlator N/2 lags x N products, each a
    multiply and an add)."""
    dof = 6 if config == "he3" else 1
    seg = 2 ** ka["S"]
    N = ka["N"]
    uni = 2 * dof + 2.0 / (seg - 1)
    if ka["enableRanlux"]:
        nskip = {0: 0, 1: 24, 2: 76, 3: 200, 4: 380}[ka["luxuaryFactor"] + 1]
        rng = uni * ((24 + nskip) / 24.0 * 3 + 8)
    else:
        rng = uni * 8
    bm = dof * 9
    # one measurement per operator run, after metroStepsPerOperatorRun sweeps of
    # (N / 2^S) * (2^S - 1) node updates per walker
    nodes_between = ka["metroStepsPerOperatorRun"] * (N // seg) * (seg - 1)
    meas = N * MEAS_OPS[config]
    if ka.get("enableCorrelator"):
        meas += len(ka.get("correlators") or ()) * (N // 2) * N * 2
    return rng + bm + 2 * POT_OPS[config] + meas / nodes_between


# DRAM bytes per fs_metropolis launch from one ncu capture of the default workload
# (dram__bytes_read.sum + dram__bytes_write.sum; profiles/fs_metropolis_he3_lm2m2_ranlux.md)
TRAFFIC_PER_LAUNCH = {"he3": 262.7e6}


def roofline_for(config, ka, node_rate, clk, default_workload=True):
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak = 4 * 32 * 152 * sm_mhz * 1e6 / 1e12            # Tera lane-ops/s
    per_node = alg_ops_per_node(config, ka)
    achieved = node_rate * per_node / 1e12
    traffic = TRAFFIC_PER_LAUNCH.get(config) if default_workload else None
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tlane-op/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_unit": "DRAM bytes per launch (ncu), against the ~250 MB of paths, RANLUX tables and "
                            "results a launch must move, plus the 16 MB potential cache: the kernel is not "
                            "memory bound",
            "alg_ops_per_node": per_node,
            "alg_basis": "the reference algorithm's lane operations per node update: RANLUX or xorshift "
                         "uniforms, Box-Muller, two potential evaluations (old and new action; with the "
                         "potential cache the old one is a cached load) and the measurements",
            "peak_basis": f"4 x 32 x 152 lanes per clock at the sampled median SM clock {sm_mhz:.0f} MHz "
                          "(MEASURED_PEAKS.json has HBM and bf16 peaks only; this kernel uses neither)"}


# ------------------------------------------------------------------ learned vs plain
def learned_study(quick=True):
    """Energy-estimator ESS/s of the plain sampler and of the learned level-1 proposal on the
    He3 workload (feynsimul_gb300.learned.ess_study), by the package's one definition
    (learned.energy_ess): per-walker energies measured after every sweep, 200 measurements
    per walker, Sokal-windowed integrated autocorrelation, ESS over the wall time of the
    measured loop; all samplers from the same equilibrated paths; training time is not
    included in ESS/s."""
    from feynsimul_gb300 import build as fb
    fb.build()
    from feynsimul_gb300.learned import ess_study
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    sysm = Lm2m2Cluster(3, 1.0)
    t0 = time.perf_counter()
    res = ess_study(sysm, sysm.beta, 256, 16384,
                    S_plain=(4, 5) if quick else (3, 4, 5, 6), S_learned=(4, 5) if quick else (4, 5, 6, 7),
                    launches=200, train_steps=1500 if quick else 3000, force_network=(4,) if quick else (4, 5, 6, 7),
                    kernel_extra=dict(enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
                                      walkersPerBlock=TUNED_WPB["he3"], minBlocksPerSM=TUNED_MIN_BLOCKS["he3"]),
                    log=lambda *a: None)
    out = {"metric": "energy ESS/s, learned vs plain sampler (He3 LM2M2 T=1K N=256 16384 walkers RANLUX)",
           "summary": res["summary"], "wall_s": time.perf_counter() - t0,
           "plain": {str(k): {kk: v[kk] for kk in ("acceptance", "tau_int_sweeps", "ess_per_s",
                                                    "node_updates_per_s")} for k, v in res["plain"].items()},
           "learned": {str(k): {kk: v[kk] for kk in ("acceptance", "tau_int_sweeps", "ess_per_s",
                                                      "node_updates_per_s", "loss_start", "loss_end",
                                                      "validation_gain_nats", "fallback")}
                       for k, v in res["learned"].items()},
           "forced": {str(k): {kk: v[kk] for kk in ("acceptance", "tau_int_sweeps", "ess_per_s", "node_updates_per_s",
                                                     "validation_gain_nats")} for k, v in res.get("forced", {}).items()}}
    if not quick:
        out["coarse_ho"] = coarse_ho_gain()
    return out


def coarse_ho_gain(N=32, S=3, beta=16.0, walkers=4096, seed=3):
    """Where the free bridge is poor -- the HO with eps = 0.5 and 8-slice segments spanning
    4 time units -- the trained network's acceptance and energy ESS per sweep against the
    plain sampler's, from the same starting paths."""
    import types
    from feynsimul_gb300.kernel import PIMCKernel
    from feynsimul_gb300.kernel_args import KernelArgs
    from feynsimul_gb300.learned import LearnedProposal, harvest_triples, sigma_level
    from feynsimul_gb300.stats import ess
    sysm = types.SimpleNamespace(DOF=1, potential="0.5 * 1.0 * x1 * x1", userCode="")

    def make(learned, sd):
        return PIMCKernel(KernelArgs(
            system=sysm, nbrOfWalkers=walkers, N=N, beta=beta, S=S, enableOperator=True,
            enableCorrelator=False, enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
            enableBins=False, nbrOfWalkersPerWorkGroup=1, enableParallelizePath=True, enableGlobalPath=False,
            enableGlobalOldPath=False, operators=("1.0 * x1 * x1",), operatorRuns=1, metroStepsPerOperatorRun=1,
            seed=sd, learnedProposal=learned))
    plain = make(False, seed)
    for _ in range(200):
        plain.run()
    s1 = sigma_level(beta, N, S, 1)
    feats, z = [], []
    for _ in range(8):
        for _ in range(10):
            plain.run()
        f, t = harvest_triples(plain.getPaths(), 1, N, S, s1, 1.0)
        feats.append(f)
        z.append(t)
    feats, z = np.concatenate(feats), np.concatenate(z)
    n_val = feats.shape[0] // 10
    model = LearnedProposal(1, s1, 1.0, seed=seed)
    model.train(feats[n_val:], z[n_val:], steps=1500, batch=4096, lr=2e-3, seed=seed)
    start = plain.getPaths()
    lrn = make(True, seed + 1)
    lrn.setLearnedProposal(model)
    out = {"workload": f"HO beta={beta} N={N} S={S} {walkers} walkers, one sweep per measurement",
           "validation_gain_nats": model.validation_gain(feats[:n_val], z[:n_val])}
    for name, k in (("plain", plain), ("learned", lrn)):
        k.setPaths(start)
        series, ar, t = [], [], 0.0
        for _ in range(300):
            k.run()
            t += k.getRunTime()
            ar.append(k.getAcceptanceRate())
            series.append(k.getOperators()[0])
        e, tau = ess(np.array(series))
        out[name] = {"acceptance": float(np.mean(ar)), "tau_int_sweeps": float(tau), "ess_per_sweep_per_walker":
                     float(e / (300 * walkers)), "ess_per_s": float(e / t)}
        k.close()
    out["ess_per_sweep_gain"] = out["learned"]["ess_per_sweep_per_walker"] / out["plain"]["ess_per_sweep_per_walker"]
    out["ess_per_s_gain"] = out["learned"]["ess_per_s"] / out["plain"]["ess_per_s"]
    return out


# ------------------------------------------------------------------ ragged batch
def batch_bench(args):
    """64 LM2M2 systems (n U{3..10}, N in {128..1024}, T U(0.5, 2) K, walkers U{1024..8192}),
    one persistent launch per step replayed from a CUDA graph, launch shape autotuned."""
    from feynsimul_gb300 import build as fb
    fb.build()
    from feynsimul_gb300.batch import BatchSampler, autotune, ragged_workload
    wl = ragged_workload(seed=0, n_systems=args.systems)
    t0 = time.perf_counter()
    tune = autotune(wl, op_runs=1, msteps=4)
    t_tune = time.perf_counter() - t0
    b = BatchSampler(wl, op_runs=1, msteps=4, block_threads=tune["block_threads"], tpw_target=tune["tpw_target"])
    for _ in range(max(3, args.warmup)):
        b.run(1)
    steps = max(3, min(args.steps, 10))
    import torch
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t = b.run(steps, graph=True)
    clk = clocks.stop()
    value = b.node_updates_per_launch * steps / t
    path_bytes = sum(w["walkers"] * w["N"] * 3 * (w["n"] - 1) * 4 for w in wl)
    # algorithmic lane operations of one launch: per system, node updates x (xorshift 8 per
    # uniform x 2 DOF uniforms + Box-Muller 9 per DOF + two LM2M2 cluster evaluations)
    ops = 0.0
    for w, sy in zip(wl, b.systems):
        n, dof = w["n"], 3 * (w["n"] - 1)
        nodes = w["walkers"] * (w["N"] >> sy.bisection_level) * ((1 << sy.bisection_level) - 1) * 4
        ops += nodes * (16 * dof + 9 * dof + 2 * lm2m2_cluster_ops(n))
    clk_mhz = clk.get("sm_mhz") or 2070.0
    peak = 4 * 32 * 152 * clk_mhz * 1e6 / 1e12
    achieved = ops * steps / t / 1e12
    out = {"metric": "path-node updates/s, ragged batch of 64 LM2M2 systems in one persistent launch",
           "value": value, "unit": "node-updates/s", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup),
           "ms_per_step": 1e3 * t / steps, "higher_is_better": True, "dtype": "f32 (u32 RNG, f64 sums)",
           "data": "synthetic, seeded", "config": {
               "workload": "64 systems: n U{3..10}, N in {128,256,512,1024}, T U(0.5,2) K, walkers U{1024..8192}, "
                           "xorshift, 4 sweeps + 1 energy measurement per step",
               "node_updates_per_step": b.node_updates_per_launch, "work_items": b.n_items, "grid": b.grid,
               "block_threads": tune["block_threads"], "tpw_target": tune["tpw_target"],
               "registers": b.registers, "smem_bytes": b.smem, "cuda_graph": True,
               "l2": f"inputs larger than L2 ({path_bytes / 1e9:.1f} GB of paths)"},
           "clocks": clk,
           "autotune": {"cached": tune["cached"], "seconds": t_tune,
                        "candidates": [{k: c.get(k) for k in ("block_threads", "tpw_target", "node_updates_per_s",
                                                              "error")} for c in tune.get("candidates", [])]},
           "gpu_launches": steps,
           "roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tlane-op/s",
                        "frac": achieved / peak, "traffic": None,
                        "alg_ops_per_node": ops / b.node_updates_per_launch,
                        "peak_basis": f"4 x 32 x 152 lanes per clock at {clk_mhz:.0f} MHz"}}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = batch_cpu_rate(wl, b, seconds=args.cpu_seconds)
    b.close()
    return out


def batch_cpu_rate(wl, b, seconds=10.0, walkers=16):
    """Node updates/s of the oracle's C restatement on the host cores for the ragged batch:
    every system run on its own (a subset of walkers, the batch's N, S, T and cadence), each
    system's CPU time per node update weighted by its node updates in the full workload."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as orc
    cores = cpu_cores()
    cfgs = []
    for w, sy in zip(wl, b.systems):
        c = b.clusters[w["n"]]
        W = min(walkers, w["walkers"])
        cfgs.append(orc.OracleConfig(
            DOF=c.DOF, potential=c.potential, userCode=c.userCode, nbrOfWalkers=W, N=w["N"], beta=1.0 / w["T"],
            S=sy.bisection_level, operatorRuns=1, metroStepsPerOperatorRun=4, enableParallelizePath=True,
            operators=(c.energyOp,), compat=False, accum=1))
    with ThreadPoolExecutor(max_workers=cores) as ex:      # gcc runs in subprocesses
        list(ex.map(orc.build, cfgs))
    per_node, real_nodes, sample_nodes, sample_t = [], [], 0, 0.0
    budget = seconds / len(cfgs)
    for w, sy, cfg in zip(wl, b.systems, cfgs):
        c = b.clusters[w["n"]]
        o = orc.OracleSampler(cfg, omp_threads=cores)
        o.paths[...] = c.initial_paths(cfg.nbrOfWalkers, w["N"], np.random.RandomState(1)).astype(np.float32)
        rs = np.random.RandomState(2)
        o.seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.seeds.shape)
        o.walker_seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape)
        seg = 2 ** sy.bisection_level
        nodes_launch = cfg.nbrOfWalkers * (w["N"] // seg) * (seg - 1) * 4
        runs, dt = 0, 0.0
        while runs < 1 or (dt < budget and runs < 1000):
            t0 = time.perf_counter()
            o.run()
            dt += time.perf_counter() - t0
            runs += 1
        per_node.append(dt / (runs * nodes_launch))
        real_nodes.append(w["walkers"] * (w["N"] // seg) * (seg - 1) * 4)
        sample_nodes += runs * nodes_launch
        sample_t += dt
    total_nodes = float(np.sum(real_nodes))
    value = total_nodes / float(np.dot(real_nodes, per_node))
    return {"value": value, "unit": "node-updates/s", "cores": cores, "kind": "port",
            "sample": f"each of the {len(cfgs)} systems with {walkers} walkers, its N, S, T and cadence "
                      f"({sample_nodes} node updates, {sample_t:.1f} s); per-system CPU time per node update "
                      f"weighted by the system's node updates in the full workload; oracle C restatement, "
                      f"OpenMP over walkers"}


def lm2m2_cluster_ops(n):
    """Lane operations of one LM2M2 cluster potential evaluation: the positions from the
    Jacobi coordinates (3n(n-1) multiply-adds) and per pair 6 for r^2 and ~40 for the pair
    potential (rsqrt, dispersion polynomial, two exponentials, the add-on cosine, selects)."""
    return 3 * n * (n - 1) + 46 * n * (n - 1) // 2


# ------------------------------------------------------------------ arms
def precision_bench(args):
    """The precision study on the 10-atom LM2M2 cluster, N = 1024, 2^20 walkers (FP32 path,
    FP64 / plain-FP32 / Kahan sums) against 2^14 walkers run FP64 everywhere from the same
    seeds (feynsimul_gb300.precision)."""
    from feynsimul_gb300.precision import precision_study
    kw = {}
    if args.walkers:
        kw["walkers"] = args.walkers
        kw["fp64_walkers"] = min(2 ** 14, args.walkers)
    if args.op_runs:
        kw["op_runs"] = args.op_runs
    if args.msteps:
        kw["msteps"] = args.msteps
    if args.minb > 0:
        kw["min_blocks"] = args.minb
    if args.S:
        kw["S"] = args.S
    import torch
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()        # sampled over the whole study: both arms' timed launches are inside
    r = precision_study(launches=max(2, args.steps), log=lambda m: print(m, file=sys.stderr), **kw)
    clk = clocks.stop()
    dof = 27
    per_node = 16 * dof + 9 * dof + 2 * lm2m2_cluster_ops(10)
    clk_mhz = clk.get("sm_mhz") or 2070.0
    peak = 4 * 32 * 152 * clk_mhz * 1e6 / 1e12
    achieved = r["fp32_node_updates_per_s"] * per_node / 1e12
    return {"roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tlane-op/s",
                         "frac": achieved / peak, "traffic": None, "alg_ops_per_node": per_node,
                         "peak_basis": f"4 x 32 x 152 lanes per clock at {clk_mhz:.0f} MHz (FP32 arm)"},
            "clocks": clk,
            "metric": "precision study: FP32-path error vs FP64-everywhere, per result",
            "value": r["fp32_node_updates_per_s"], "unit": "node-updates/s (FP32 path, study sums)",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f32 path, f64/f32/kahan sums",
            "data": "synthetic, seeded", "config": {"workload": r["workload"]}, "study": r}


def _compact_merge(m):
    """The replica merge of every accumulator, shortened for the JSON line: histogram and
    bin counts as totals."""
    out = {k: v for k, v in m.items() if k not in ("histogram_counts", "bin_counts")}
    if "histogram_counts" in m:
        out["histogram_total_counts"] = int(np.sum(m["histogram_counts"]))
    if "bin_counts" in m:
        out["bin_total_counts"] = int(np.sum(m["bin_counts"]))
    return out


def oracle_cpu_ess(sysm, ka, extra, paths, launches=200, burn=10, walkers=64):
    """The CPU baseline of the energy ESS/s: the oracle's C restatement on the host cores with
    the same definition as learned.energy_ess (one measurement per walker after every sweep,
    Sokal window, ESS over the wall time of the measured loop incl. the per-walker energy
    reduction), on `walkers` walkers started from the given equilibrated paths."""
    from oracle import oracle as orc
    from feynsimul_gb300.stats import ess
    cores = cpu_cores()
    W = min(walkers, ka["nbrOfWalkers"])
    cfg = orc.OracleConfig(
        DOF=sysm.DOF, potential=sysm.potential, userCode=sysm.userCode, nbrOfWalkers=W, N=ka["N"],
        beta=ka["beta"], S=ka["S"], operatorRuns=1, metroStepsPerOperatorRun=1, nbrOfWalkersPerWorkGroup=1,
        enableParallelizePath=True, enableRanlux=ka["enableRanlux"], luxuaryFactor=ka.get("luxuaryFactor", 2),
        ranluxIntMax=ka.get("ranluxIntMax", 2 ** 32 - 1), operators=ka["operators"], compat=False, accum=1)
    o = orc.OracleSampler(cfg, omp_threads=cores)
    o.paths[...] = paths[:W]
    if ka["enableRanlux"]:
        o.init_ranlux_rows(o.ranlux_tab, (np.uint64(777) << np.uint64(32)) + np.arange(o.ranlux_tab.shape[0], dtype=np.uint64))
        o.init_ranlux_rows(o.group_tab, (np.uint64(778) << np.uint64(32)) + np.arange(o.group_tab.shape[0], dtype=np.uint64))
    else:
        rs = np.random.RandomState(3)
        o.seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.seeds.shape)
        o.walker_seeds[...] = rs.randint(0, 2 ** 31 - 1, size=o.walker_seeds.shape)
    T = ka["N"] // 2 ** ka["S"]
    for _ in range(burn):
        o.run()
    series = []
    t0 = time.perf_counter()
    for _ in range(launches):
        o.run()
        series.append(o.op_means.reshape(W, T, -1)[:, :, 0].mean(axis=1))
    wall = time.perf_counter() - t0
    e, tau = ess(np.array(series))
    return {"value": e / wall, "unit": "effective energy samples/s", "cores": cores, "kind": "port",
            "tau_int_sweeps": float(tau), "sample": f"{W} walkers x {launches} sweeps, one measurement per sweep "
            f"({wall:.1f} s), oracle C restatement, OpenMP over walkers"}


def run_gb300(args, rank, world):
    from feynsimul_gb300 import build as fb
    fb.build()
    import torch
    from feynsimul_gb300.kernel import PIMCKernel
    from feynsimul_gb300.kernel_args import KernelArgs

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    setup = he3_setup if args.config == "he3" else ho_setup
    sysm, ka, extra, workload = setup(**workload_overrides(args))
    minb = args.minb if args.minb >= 0 else TUNED_MIN_BLOCKS.get(args.config, 0)
    wpb = args.wpb if args.wpb > 0 else TUNED_WPB.get(args.config, 0)
    from feynsimul_gb300.replicas import ReplicaGroup, replica_seed
    group = ReplicaGroup()
    pc = {"auto": None, "shared": True, "device": "device", "off": False}[args.potential_cache]
    ka_obj = KernelArgs(system=sysm, seed=replica_seed(1000, rank), walkersPerBlock=wpb,
                        minBlocksPerSM=minb, potentialCache=pc, **extra, **ka)
    k = PIMCKernel(ka_obj)
    paths0 = initial_paths(sysm, ka, replica_seed(17, rank))
    k.setPaths(paths0)
    if ka["enableRanlux"]:
        k.initRanlux()
        k.groupInitRanlux()
    info = k.getInfo()
    nodes = node_updates_per_run(ka)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        k.run()
    # ---- device-resident throughput ----
    clocks = ClockSampler(dev)
    clocks.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        flush.zero_()  # 512 MiB write: L2 (129 MB) holds nothing of the previous launch
        torch.cuda.synchronize()
        k.run()
        times.append(k.getRunTime())
    torch.cuda.synchronize()
    clk = clocks.stop()
    t_dev = group.max(float(np.sum(times)))
    value = nodes * args.steps * world / t_dev
    ms_per_step = 1e3 * t_dev / args.steps

    # ---- end to end through the public API, host buffers ----
    # Each step: this step's input paths copied in from pinned host memory, the sweeps, the
    # paths copied back (PIMCKernel.runHost: chunks of walkers pipelined over three
    # streams), and the per-walker operator means read back and reduced on the host.
    host_paths = np.ascontiguousarray(k.getPaths())
    try:
        k.pinHost(host_paths)
        pinned = True
    except Exception:
        pinned = False
    energies = []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        k.runHost(host_paths, out=host_paths, chunks=args.chunks)
        ops = k.getOperators()          # D2H: per-thread operator means, reduced per walker
        energies.append(ops[0])
    t_e2e = group.max(time.perf_counter() - t0)
    if pinned:
        try:
            k.unpinHost(host_paths)
        except Exception:
            pass
    e2e_value = nodes * args.steps * world / t_e2e
    h2d = host_paths.nbytes
    d2h = ops.nbytes + host_paths.nbytes   # per-walker operator means + the paths

    series = np.array(energies)  # [steps, walkers]

    # ---- energy ESS/s (learned.energy_ess): one measurement per walker after every sweep,
    # 200 measurements, ESS over the wall time of that loop, from the equilibrated paths ----
    ess_rec = None
    if args.config == "he3" and not args.no_ess:
        from feynsimul_gb300.learned import energy_ess
        ka_e = dict(ka, operatorRuns=1, metroStepsPerOperatorRun=1)
        ke = PIMCKernel(KernelArgs(system=sysm, seed=replica_seed(2000, rank), walkersPerBlock=wpb,
                                   minBlocksPerSM=minb, potentialCache=pc, **extra, **ka_e))
        ke.setPaths(host_paths)
        if ka["enableRanlux"]:
            ke.initRanlux()
            ke.groupInitRanlux()
        m = energy_ess(ke, launches=args.ess_launches, burn=10)
        ser = m.pop("series")
        ke.close()
        ess_rec = dict(m, ess=group.sum(m["ess"]), ess_per_s=group.sum(m["ess"]) / group.max(m["wall_s"]),
                       unit="effective energy samples/s", energy_mean=float(ser.mean()),
                       definition="learned.energy_ess: per-walker virial energy after every sweep, Sokal "
                                  "window (c=5), ESS / wall time of the measured loop incl. reads")

    # ---- roofline: the sweep is bound by instruction issue (see roofline_for) ----
    roof = roofline_for(args.config, ka, value / world, clk,
                        default_workload=not (args.walkers or args.op_runs or args.msteps or args.S))

    result = {
        "metric": "path-node updates/s (plain Metropolis-bisection sampler)",
        "value": value, "unit": "node-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (u32 RNG, f64 sums)",
        "data": "synthetic, seeded",
        "config": bench_config(workload, ka),
        "timing": {"l2": "flushed between launches (512 MiB write)", "parallelism": f"replicas x{world}"},
        "launch": {"walkers_per_block": int(info.walkers_per_block), "registers": int(info.registers),
                   "smem_bytes": int(info.smem_bytes), "grid": int(info.grid_blocks),
                   "potential_cache": {0: "none", 1: "shared", 3: "device"}.get(int(info.potential_cache))},
        "e2e": {"value": e2e_value, "unit": "node-updates/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "pinned": pinned, "api": "PIMCKernel.runHost + getOperators",
                "chunks": k.lastChunks},
        "energy_ess": ess_rec,
        "energy_mean": float(series[series.shape[0] // 2:].mean()),
        "energy_all_replicas": group.merge(series[series.shape[0] // 2:].mean(axis=0)),
        "accumulators_all_replicas": _json_safe(_compact_merge(group.merge_kernel(k))),
        "acceptance_rate": float(k.getAcceptanceRate()),
        "gpu_launches": args.steps * (2 + k.lastChunks),  # sweeps, pipelined chunks, walker reductions
        "roofline": roof, "clocks": clk,
    }
    k.close()
    return result, (sysm, ka, extra, host_paths)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="he3", choices=["he3", "ho", "learned", "batch", "precision"])
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain ESS study")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--walkers", type=int, default=0, help="override the walker count (small cases)")
    ap.add_argument("--op-runs", type=int, default=0, help="override operatorRuns per launch")
    ap.add_argument("--msteps", type=int, default=0, help="override metroStepsPerOperatorRun")
    ap.add_argument("--S", type=int, default=0, help="override the bisection level")
    ap.add_argument("--wpb", type=int, default=0, help="walkers per thread block (0 = automatic)")
    ap.add_argument("--minb", type=int, default=-1, help="thread blocks per SM to compile for (-1 = tuned default)")
    ap.add_argument("--chunks", type=int, default=0,
                    help="walker chunks pipelined in the e2e step (0 = automatic, 1 = no overlap)")
    ap.add_argument("--systems", type=int, default=64, help="batch config: number of systems (small profiling cases)")
    ap.add_argument("--no-ess", action="store_true", help="skip the energy ESS/s measurement")
    ap.add_argument("--ess-launches", type=int, default=200, help="measurements per walker of the ESS loop")
    ap.add_argument("--no-batch", action="store_true", help="skip the ragged-batch sub-record of the default run")
    ap.add_argument("--no-ho", action="store_true", help="skip the harmonic-oscillator sub-record of the default run")
    ap.add_argument("--potential-cache", default="auto", choices=["auto", "shared", "device", "off"],
                    help="he3 / ho configs: where V of every slice is kept between moves (auto = the library's choice)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        setup = he3_setup if args.config == "he3" else ho_setup
        sysm, ka, extra, workload = setup(**workload_overrides(args))
        vals = []
        for _ in range(args.warmup):
            reference_cpu_rate(args.config, sysm, ka, extra, seconds=1.0)
        t_all = []
        for _ in range(args.steps):
            cb = reference_cpu_rate(args.config, sysm, ka, extra, seconds=max(1.0, 60.0 / max(1, args.steps)))
            vals.append(cb["value"])
            t_all.append(cb["seconds"])
        v = float(np.median(vals))
        out = {"impl": "reference", "metric": "path-node updates/s (plain Metropolis-bisection sampler)",
               "value": v, "unit": "node-updates/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": 1e3 * float(np.mean(t_all)),
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic, seeded", "config": bench_config(workload, ka),
               "cpu_baseline": dict(cb, value=v),
               "e2e": {"value": v, "unit": "node-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "note": "no OpenCL CPU platform is installed; the reference's own kernel.c (as its kernel.py "
                       "generates it) is compiled for the host and its work-groups run on every host thread "
                       "(cpu_baseline.kind 'reference'), or, where that sample is absent, the oracle's C "
                       "restatement of the reference sweep (kind 'port'); a step is a bounded sample of the "
                       "workload (ms_per_step is its timed part)"}
        print(json.dumps(out))
        return

    if args.config == "batch":
        if rank == 0:
            print(json.dumps(batch_bench(args)))
        return
    if args.config == "learned":
        if rank == 0:
            print(json.dumps(learned_study(quick=False)))
        return
    if args.config == "precision":
        if rank == 0:
            print(json.dumps(precision_bench(args)))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    result, (sysm, ka, extra, paths_eq) = run_gb300(args, rank, world)
    if rank == 0:
        if args.config == "he3" and not args.no_learned:
            result["learned_vs_plain"] = learned_study(quick=True)["summary"]
        if not args.no_cpu_baseline:
            result["cpu_baseline"] = reference_cpu_rate(args.config, sysm, ka, extra, seconds=args.cpu_seconds)
            if result.get("energy_ess"):
                result["energy_ess"]["cpu_baseline"] = oracle_cpu_ess(sysm, ka, extra, paths_eq,
                                                                      launches=args.ess_launches)
        if args.config == "he3" and not args.no_batch:
            # the ragged batch (64 LM2M2 systems in one persistent launch) as a sub-record
            bargs = argparse.Namespace(**vars(args))
            bargs.steps, bargs.warmup, bargs.cpu_seconds = min(args.steps, 5), 3, min(args.cpu_seconds, 6.0)
            br = batch_bench(bargs)
            result["ragged_batch"] = {k: br[k] for k in ("metric", "value", "unit", "ms_per_step", "steps",
                                                         "roofline", "clocks", "config", "gpu_launches",
                                                         "cpu_baseline") if k in br}
        if args.config == "he3" and not args.no_ho and world == 1:
            # config 1 (1D HO, correlator every sweep) as a sub-record, same timing rules
            hargs = argparse.Namespace(**vars(args))
            hargs.config, hargs.no_ess = "ho", True
            # a launch is ~0.14 ms: 3000 of them give the clock sampler (200 ms period) a
            # timed region to sample
            hargs.steps = max(args.steps, 3000)
            hargs.walkers = hargs.op_runs = hargs.msteps = hargs.S = hargs.wpb = 0
            hargs.minb = -1
            hr, hctx = run_gb300(hargs, 0, 1)
            hrec = {k: hr[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "config", "launch",
                                       "e2e", "roofline", "clocks", "gpu_launches", "acceptance_rate")}
            if not args.no_cpu_baseline:
                hrec["cpu_baseline"] = oracle_cpu_rate(*hctx[:3], seconds=min(args.cpu_seconds, 4.0))
            result["harmonic_oscillator"] = hrec
        print(json.dumps(_json_safe(result)))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
