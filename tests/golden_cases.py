"""Shared helpers for the golden fixtures produced by tests/golden/make_golden.py."""
import ast
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

HO = dict(DOF=1, potential="0.5 * 1.0 * x1 * x1",
          userCode="FLOAT_TYPE sqr(FLOAT_TYPE x){return x*x;}")


def sweep_cases():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "sweep_*.npz")))


def load_sweep(name):
    z = np.load(os.path.join(GOLDEN, f"sweep_{name}.npz"))
    rec = {k: z[k] for k in z.files}
    ka = ast.literal_eval(str(rec.pop("config")))
    return ka, rec


def load_ranlux():
    z = np.load(os.path.join(GOLDEN, "ranlux_streams.npz"))
    return {k: z[k] for k in z.files}


def oracle_config(ka, compat=True, accum=0):
    from oracle.oracle import OracleConfig
    return OracleConfig(
        DOF=HO["DOF"], potential=HO["potential"], userCode=HO["userCode"],
        nbrOfWalkers=ka["nbrOfWalkers"], N=ka["N"], beta=ka["beta"], S=ka["S"],
        operatorRuns=ka["operatorRuns"], metroStepsPerOperatorRun=ka["metroStepsPerOperatorRun"],
        nbrOfWalkersPerWorkGroup=ka["nbrOfWalkersPerWorkGroup"],
        enableParallelizePath=ka["enableParallelizePath"], enableRanlux=ka["enableRanlux"],
        luxuaryFactor=ka.get("luxuaryFactor", 2), ranluxIntMax=ka.get("ranluxIntMax", 2 ** 32 - 1),
        enableDouble=ka["enableDouble"],
        operators=tuple(ka["operators"]) if ka["enableOperator"] else (),
        correlators=tuple(ka["correlators"]) if ka["enableCorrelator"] else (),
        enableBins=ka["enableBins"], xMin=ka["xMin"], xMax=ka["xMax"],
        binResolutionPerDOF=ka["binResolutionPerDOF"], compat=compat, accum=accum,
        enableBisection=ka.get("enableBisection", True), enablePathShift=ka.get("enablePathShift", False),
        enableSingleNodeMove=ka.get("enableSingleNodeMove", False), alpha=ka.get("alpha") or 0.0,
        PSAlpha=ka.get("PSAlpha") or 0.0)
