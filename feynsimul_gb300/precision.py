"""Precision study: FP32 path, action and potential arithmetic with the operator and
correlator running sums kept three ways (plain FP32, Kahan-compensated FP32, FP64), each
compared against an FP64-everywhere run of the same seeds.

No counterpart in the reference, whose sums are FLOAT_TYPE throughout (kernel.c:622,
:784-788) and whose ENABLE_DOUBLE build (kernel.c:40-59) is the FP64-everywhere arm here.

Workload: an n-atom He-4 cluster with the LM2M2 pair potential (physical_systems.lm2m2)
in mass-scaled Jacobi coordinates, N slices, W walkers, xorshift generator, paths in
device memory (enableGlobalPath: a 10-atom, 1024-slice FP64 walker is 221 KB).  The
starting paths are classical cluster configurations tiled over the walkers on the device
(walker w starts from template w % n_templates).

Per result (the virial energy estimator and the correlator of the squared hyperradius
rho^2 = sum_i x_i^2) the study reports:

1. accumulation error, on one trajectory: the plain-FP32 and Kahan sums against the FP64
   sum of the same per-slice FP32 values (relative error of the ensemble mean; for the
   energy also the worst walker);
2. arithmetic error: the first ``fp64_walkers`` walkers run again with FP64 paths,
   action, potential and sums from the same seeds and starting paths.  The two runs
   start equal and part as rounding changes accept decisions, so they are compared
   statistically: for the energy by the paired per-walker difference and its standard
   error, for the correlator by the difference of walker means against the combined
   standard error.

The FP64-everywhere sweep itself is checked against the CPU oracle's FP64 build in the
tests.
"""
from __future__ import annotations

import time

import numpy as np


def hyperradius2(dof):
    return " + ".join(f"x{i + 1} * x{i + 1}" for i in range(dof))


def _kernel(sysm, walkers, N, S, op_runs, msteps, double, accumulation, seed, fast_math, min_blocks=0):
    from .kernel import PIMCKernel
    from .kernel_args import KernelArgs
    ka = KernelArgs(system=sysm, nbrOfWalkers=walkers, N=N, beta=sysm.beta, S=S, enableOperator=True,
                    enableCorrelator=True, enableBisection=True, enablePathShift=False,
                    enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
                    enableParallelizePath=True, enableGlobalPath=True, enableGlobalOldPath=False,
                    enableDouble=double, operators=(sysm.energyOp,), correlators=(hyperradius2(sysm.DOF),),
                    operatorRuns=op_runs, metroStepsPerOperatorRun=msteps, accumulation=accumulation,
                    fastMath=fast_math, seed=seed, minBlocksPerSM=min_blocks)
    return PIMCKernel(ka)


def precision_study(n_atoms=10, N=1024, walkers=2 ** 20, T=1.0, S=2, op_runs=2, msteps=2, launches=8,
                    fp64_walkers=2 ** 14, n_templates=256, seed=2024, fast_math=True, lags=(0, 1, 2, 4, 8),
                    burn_in=2, log=None, min_blocks=2):
    """Run the study (``burn_in`` launches of both arms before the measured ones, after
    which the accumulators are zeroed); returns a dict of results (JSON-serialisable)."""
    from .physical_systems.lm2m2 import Lm2m2Cluster
    sysm = Lm2m2Cluster(n_atoms, T)
    fp64_walkers = min(fp64_walkers, walkers)
    n_templates = min(n_templates, fp64_walkers)
    if fp64_walkers % n_templates or walkers % n_templates:
        raise ValueError("walker counts must be multiples of n_templates")
    rng = np.random.RandomState(seed)
    tmpl = sysm.initial_paths(n_templates, N, rng, noise=0.0)

    t0 = time.time()
    k32 = _kernel(sysm, walkers, N, S, op_runs, msteps, False, "study", seed, fast_math, min_blocks)
    k64 = _kernel(sysm, fp64_walkers, N, S, op_runs, msteps, True, "fp64", seed, fast_math)
    setup_s = time.time() - t0
    k32.setPathsTiled(tmpl.astype(np.float32))
    k64.setPathsTiled(tmpl.astype(np.float64))
    tpw = N >> S
    k64.setSeeds(k32.getSeeds()[:fp64_walkers * tpw + 1])
    k64.setWalkerSeeds(k32.getWalkerSeeds()[:fp64_walkers])

    for it in range(burn_in):
        k32.run()
        k64.run()
    k32.zeroAccumulators()
    k64.zeroAccumulators()
    e32 = np.zeros((3, walkers))
    e64 = np.zeros(fp64_walkers)
    t32 = t64 = 0.0
    acc32 = acc64 = 0
    for it in range(launches):
        k32.run()
        t32 += k32.getRunTime()
        e32 += k32.getOperatorsStudy()[:, 0, :]
        acc32 += int(k32.getAccepts().sum(dtype=np.int64))
        k64.run()
        t64 += k64.getRunTime()
        e64 += k64.getOperators()[0]
        acc64 += int(k64.getAccepts().sum(dtype=np.int64))
        if log:
            log(f"launch {it}: fp32 {t32:.2f} s, fp64 {t64:.2f} s")
    e32 /= launches
    e64 /= launches

    moves32 = walkers * tpw * op_runs * msteps * launches
    moves64 = fp64_walkers * tpw * op_runs * msteps * launches
    nodes_per_launch = walkers * tpw * ((1 << S) - 1) * op_runs * msteps

    def rel(a, b):
        return float(abs(a - b) / max(abs(b), 1e-300))

    ref = e32[2]
    energy = {
        "fp64_sum_mean_K": float(ref.mean()),
        "fp32_sum_rel_err": rel(e32[0].mean(), ref.mean()),
        "kahan_sum_rel_err": rel(e32[1].mean(), ref.mean()),
        "fp32_sum_worst_walker_rel_err": float(np.max(np.abs(e32[0] - ref) / np.maximum(np.abs(ref), 1e-300))),
        "kahan_sum_worst_walker_rel_err": float(np.max(np.abs(e32[1] - ref) / np.maximum(np.abs(ref), 1e-300))),
    }
    d = ref[:fp64_walkers] - e64
    se = float(d.std(ddof=1) / np.sqrt(fp64_walkers))
    se_u = float(np.sqrt((ref[:fp64_walkers].var(ddof=1) + e64.var(ddof=1)) / fp64_walkers))
    energy.update({
        "fp64_everywhere_mean_K": float(e64.mean()),
        "fp32_path_mean_same_walkers_K": float(ref[:fp64_walkers].mean()),
        "diff_K": float(d.mean()),
        "diff_rel": rel(ref[:fp64_walkers].mean(), e64.mean()),
        # statistical error of either estimate: is the FP32-path result within its error
        # bar of the FP64 one?
        "unpaired_se_K": se_u, "z_unpaired": float(d.mean() / se_u) if se_u > 0 else 0.0,
        # paired per-walker difference: the runs share seeds and starting paths, so this
        # resolves the systematic FP32 arithmetic error far below the statistical error
        "paired_se_K": se, "paired_z": float(d.mean() / se) if se > 0 else 0.0,
    })

    m_all, s_all = k32.getCorrelatorMoments()            # (3, 1, N/2)
    m_sub, s_sub = k32.getCorrelatorMoments((0, fp64_walkers))
    m64, s64 = k64.getCorrelatorMoments()                 # (1, N/2)
    cref = m_all[2, 0]
    rel_f = np.abs(m_all[0, 0] - cref) / np.abs(cref)
    rel_k = np.abs(m_all[1, 0] - cref) / np.abs(cref)
    z = (m_sub[2, 0] - m64[0]) / np.sqrt(s_sub[2, 0] ** 2 + s64[0] ** 2)
    sums_per_lag = N * op_runs * launches
    corr = {
        "sums_per_lag_per_walker": int(sums_per_lag),
        "fp64_sum": {str(l): float(cref[l]) for l in lags},
        "fp32_sum_rel_err": {str(l): float(rel_f[l]) for l in lags},
        "kahan_sum_rel_err": {str(l): float(rel_k[l]) for l in lags},
        "fp32_sum_rel_err_max_over_lags": float(rel_f.max()),
        "kahan_sum_rel_err_max_over_lags": float(rel_k.max()),
        "fp64_everywhere": {str(l): float(m64[0][l]) for l in lags},
        "z_vs_fp64_everywhere": {str(l): float(z[l]) for l in lags},
        "max_abs_z_over_lags": float(np.max(np.abs(z))),
    }
    out = {
        "workload": f"LM2M2 He-4 cluster n={n_atoms} (DOF {sysm.DOF}), N={N}, T={T} K, S={S}, "
                    f"{walkers} walkers (FP32 path) + {fp64_walkers} (FP64 everywhere), xorshift, "
                    f"op_runs {op_runs} x msteps {msteps} x {launches} launches after {burn_in} burn-in launches",
        "fast_math": bool(fast_math),
        "energy": energy,
        "correlator_rho2": corr,
        "fp32_node_updates_per_s": nodes_per_launch * launches / t32,
        "fp64_node_updates_per_s": fp64_walkers * tpw * ((1 << S) - 1) * op_runs * msteps * launches / t64,
        "fp32_seconds": t32, "fp64_seconds": t64, "setup_seconds": setup_s,
        "acceptance_fp32": acc32 / moves32, "acceptance_fp64": acc64 / moves64,
    }
    k32.close()
    k64.close()
    return out
