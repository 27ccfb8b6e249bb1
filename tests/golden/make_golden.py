"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference's source tree exists:

    python tests/golden/make_golden.py

It compiles the reference's kernel.c (as produced by its kernel.py) and its vendored
RANLUXCL header on the CPU (oracle/build_ref.py) and records inputs and outputs:

* ``ranlux_streams.npz``: RANLUXCL uniforms and final 28-word states for luxury levels
  0-4 and p=124, FP32 and FP64 variants (pyopencl-ranluxcl.cl:384-557, :597-725, :893-920);
* ``lm2m2_ref.npz``: the reference's LM2M2 pair potential and derivative routine
  (physical_systems/lm2m2.h) on a grid of pair distances;
* ``plugins_ref.npz``: the reference's three- and four-atom plugin expressions
  (physical_systems/lm2m2_3part.py, lm2m2_4part.py) at seeded coordinates;
* ``sweep_<case>.npz``: initial paths and seed tables, and after each of two
  ``metropolis`` launches: paths, accept counts, seed / RANLUX tables, operator means,
  correlator sums and histogram bins (kernel.c:514-837).

The fixtures hold numbers only (no reference source text).  The plugin used is the
1D harmonic oscillator V = 0.5*k*x^2 with the virial operator k*x^2
(FeynSimul/physical_systems/harm_osc.py:46-53), written out in ``CASES`` below.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_ref as br  # noqa: E402

HO = dict(DOF=1, potential="0.5 * 1.0 * x1 * x1",
          userCode="FLOAT_TYPE sqr(FLOAT_TYPE x){return x*x;}")

BASE = dict(nbrOfWalkers=8, N=16, beta=10.0, S=2, enableOperator=True, enableCorrelator=True,
            enableBisection=True, enablePathShift=False, enableSingleNodeMove=False,
            enableBins=True, nbrOfWalkersPerWorkGroup=2, enableParallelizePath=True,
            enableGlobalPath=True, enableGlobalOldPath=False, enableDouble=False,
            enableRanlux=False, operators=("1.0 * x1 * x1", "x1"),
            correlators=("x1", "x1*x1"), operatorRuns=3, metroStepsPerOperatorRun=5,
            xMin=-3.0, xMax=3.0, binResolutionPerDOF=10)

CASES = {
    "xorshift_parallel": dict(BASE),
    "xorshift_parallel_wpg1_s3": dict(BASE, nbrOfWalkers=6, N=32, S=3, nbrOfWalkersPerWorkGroup=1),
    "xorshift_walker": dict(BASE, enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1),
    "xorshift_parallel_double": dict(BASE, enableDouble=True),
    "ranlux_parallel_lux2": dict(BASE, enableRanlux=True, luxuaryFactor=2, ranluxIntMax=2 ** 32 - 1,
                                 nbrOfWalkersPerWorkGroup=1, nbrOfWalkers=4),
    "ranlux_walker_lux0": dict(BASE, enableRanlux=True, luxuaryFactor=0, ranluxIntMax=2 ** 31 - 1,
                               enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1,
                               nbrOfWalkers=4, S=3),
    "xorshift_parallel_s1_big": dict(BASE, nbrOfWalkers=4, N=64, S=1, nbrOfWalkersPerWorkGroup=4,
                                     operatorRuns=2, metroStepsPerOperatorRun=3),
    # walker-mode move types (kernel.c:407-473, :640-705)
    "xorshift_walker_moves": dict(BASE, enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1,
                                  enablePathShift=True, PSAlpha=0.7, enableSingleNodeMove=True, alpha=0.9,
                                  metroStepsPerOperatorRun=7),
    "xorshift_walker_snm_only": dict(BASE, enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1,
                                     enableBisection=False, enableSingleNodeMove=True, alpha=1.2),
    "ranlux_walker_moves": dict(BASE, enableRanlux=True, luxuaryFactor=1, ranluxIntMax=2 ** 32 - 1,
                                enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1, nbrOfWalkers=4,
                                enablePathShift=True, PSAlpha=0.5, enableSingleNodeMove=True, alpha=0.7),
    "xorshift_walker_shift_double": dict(BASE, enableParallelizePath=False, nbrOfWalkersPerWorkGroup=1,
                                         enableDouble=True, enablePathShift=True, PSAlpha=0.6),
}


def make_ranlux():
    seeds = np.array([1, 12345, 2 ** 31 - 5, 987654321123, 0xDEADBEEFCAFE], np.uint64)
    out = {"seeds": seeds}
    for lux in (0, 1, 2, 3, 4, 124):
        s32, st = br.ref_ranlux_streams(lux, seeds, 100)
        s64, _ = br.ref_ranlux_streams(lux, seeds[:2], 40, double=True)
        st[:, 25] = 0  # padding word, uninitialised in the reference
        out[f"f32_lux{lux}"] = s32
        out[f"state_lux{lux}"] = st
        out[f"f64_lux{lux}"] = s64
    np.savez_compressed(os.path.join(HERE, "ranlux_streams.npz"), **out)


def make_sweep(name, ka):
    system = types.SimpleNamespace(**HO)
    r = br.RefKernel(ka, system, np_seed=11)
    k = r.k
    rng = np.random.RandomState(5)
    p0 = (rng.randn(*k._paths.arr.shape) * 0.3).astype(k._paths.arr.dtype)
    k._paths.arr[...] = p0
    rec = {"paths0": p0.copy()}
    if ka["enableRanlux"]:
        rec["seeds_ranlux"] = k._seeds.arr.copy()
        rec["group_seeds"] = k._groupSeeds.arr.copy()
        r.init_ranlux()
        r.group_init_ranlux()
        rec["ranlux_tab0"] = k._ranluxcltab.arr.reshape(-1, 28).copy()
        rec["group_tab0"] = k._groupRanluxcltab.arr.reshape(-1, 28).copy()
    else:
        rec["seeds0"] = k._seeds.arr.copy()
    for it in range(2):
        r.run()
        rec[f"paths{it + 1}"] = k._paths.arr.copy()
        rec[f"accepts{it + 1}"] = k._accepts.arr.copy()
        rec[f"ops{it + 1}"] = k._operatorValues.arr.copy()
        rec[f"cor{it + 1}"] = k._correlatorValues.arr.copy()
        rec[f"bins{it + 1}"] = k._binCounts.arr.ravel().copy()
        if ka["enableRanlux"]:
            rec[f"ranlux_tab{it + 1}"] = k._ranluxcltab.arr.reshape(-1, 28).copy()
            rec[f"group_tab{it + 1}"] = k._groupRanluxcltab.arr.reshape(-1, 28).copy()
        else:
            rec[f"seeds{it + 1}"] = k._seeds.arr.copy()
    for key in list(rec):
        if "tab" in key:
            rec[key][:, 25] = 0  # padding word
    cfg = {k2: v for k2, v in ka.items()}
    rec["config"] = np.array(repr(cfg))
    np.savez_compressed(os.path.join(HERE, f"sweep_{name}.npz"), **rec)


def make_lm2m2():
    """``lm2m2_ref.npz``: the reference's pair potential lm2m2sqrt(r^2) and its derivative
    routine dlm2m2sqrtdr(r^2) (physical_systems/lm2m2.h), built as-is in FP64 and FP32, on a
    grid of r from 0.3 to 20 Angstrom."""
    libs = br.lm2m2_header_lib()
    r = np.concatenate([np.linspace(0.3, 2.5, 221), np.linspace(2.5, 6.0, 3501)[1:], np.linspace(6.0, 20.0, 141)[1:]])
    out = {"r": r}
    for ft, dt in (("double", np.float64), ("float", np.float32)):
        sr = np.ascontiguousarray((r * r).astype(dt))
        v, dv = np.zeros_like(sr), np.zeros_like(sr)
        libs[ft].ref_lm2m2(sr.ctypes.data, v.ctypes.data, dv.ctypes.data, len(sr))
        out[f"r2_{ft}"], out[f"v_{ft}"], out[f"dv_{ft}"] = sr, v, dv
    np.savez_compressed(os.path.join(HERE, "lm2m2_ref.npz"), **out)


PLUGIN_ATTRS = ("potential", "energyOp", "meanSquaredRadiusOp", "meanRadiusOp", "meanSquaredAtomDistOp")


def make_plugins():
    """``plugins_ref.npz``: the reference's three- and four-atom LM2M2 plugins
    (physical_systems/lm2m2_3part.py, lm2m2_4part.py): potential, virial energy operator and
    radius operators evaluated in FP64 from their own C strings at seeded coordinates."""
    rng = np.random.RandomState(77)
    out = {}
    for module, cls, dof in (("lm2m2_3part", "Lm2m2_3part", 6), ("lm2m2_4part", "Lm2m2_4part", 9)):
        x = rng.normal(0.0, 3.0, size=(96, dof))
        out[f"{module}_x"] = x
        out[f"{module}_values"] = br.reference_plugin_values(module, cls, PLUGIN_ATTRS, x)
    np.savez_compressed(os.path.join(HERE, "plugins_ref.npz"), **out)


def main():
    if not br.reference_available():
        raise SystemExit("reference tree not present; fixtures are generated where it is")
    only = sys.argv[1:]
    if not only:
        make_ranlux()
        make_lm2m2()
    if not only or "plugins" in only:
        make_plugins()
    for name, ka in CASES.items():
        if only and name not in only:
            continue
        make_sweep(name, ka)
        print("wrote", name)


if __name__ == "__main__":
    main()
