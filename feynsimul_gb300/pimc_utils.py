"""The reference's run loop, modN (FeynSimul/pimc_utils.py:28-355), on the GB300 engine.

Same signature, file layout and formats:

* results/<experimentName>/<YYYY-MM-DD/HH.MM.SS>/data.tsv: ``#Beta`` header, a column
  header, then per run ``N, time, pathChanges, AR, S`` and every walker's operator means,
  operator-major (``_output``, pimc_utils.py:287-355);
* ``pathsN<N>episode<k>``: tab-separated paths, one walker per row, every
  ``savePathsInterval`` runs and at the end of each N (:246-252);
* ``timestamps``: one line per N (:263-265); ``systemInfo`` (empty, :156-158);
* N doubling with linear interpolation of the paths (:207-224), S clamped to
  ``[ceil(log2(WPG*N/maxWGSize)), log2 N]`` (:171-176) and adapted from the acceptance rate
  (:272-279); resume from a path file (:129-141, :199-205).

Changes: S adaptation is bounded by log2 of the next N (the reference uses a leaked loop
variable there, :275-277, which is undefined on resume under Python 3); the periodic
``_queue.finish()`` (:236-238) is kept; and ``checkpointEvery`` (new) writes a binary
checkpoint (paths, RNG tables, running sums, run counters; ``checkpoint.npz``) from which
``resumeCheckpoint`` continues bit for bit.
"""
from __future__ import annotations

import copy
import csv
import os
from datetime import datetime
from time import time

import numpy as np

from .kernel import PIMCKernel
from .kernel_args import KernelArgs  # noqa: F401  (re-exported like the reference)


def interpolate_paths(old_paths, dof, n_old):
    """Double the slices of (walkers, DOF*n_old) paths: old nodes on even slices, midpoints of
    periodic neighbours on odd slices (pimc_utils.py:207-224)."""
    old = np.asarray(old_paths, dtype=np.float64).reshape(old_paths.shape[0], dof, n_old)
    new = np.empty((old.shape[0], dof, 2 * n_old), np.float64)
    new[:, :, 0::2] = old
    new[:, :, 1::2] = 0.5 * (old + np.roll(old, -1, axis=2))
    return new.reshape(old.shape[0], dof * 2 * n_old)


def straight_paths(startXList, walkers, dof, N):
    """Constant paths at startXList[walker][dof] (pimc_utils.py:192-198)."""
    x = np.asarray(startXList, dtype=np.float64).reshape(walkers, dof)
    return np.repeat(x[:, :, None], N, axis=2).reshape(walkers, dof * N)


def read_paths_csv(filename, walkers, width):
    rows = []
    with open(filename) as f:
        for row in csv.reader(f, delimiter="\t"):
            if row:
                rows.append([float(v) for v in row if v != ""])
    a = np.array(rows, dtype=np.float64)
    if a.shape != (walkers, width):
        raise ValueError(f"{filename}: expected {walkers} rows of {width} values, got {a.shape}")
    return a


def write_paths_csv(filename, paths):
    with open(filename, "w", newline="") as f:
        w = csv.writer(f, delimiter="\t")
        for p in paths:
            w.writerow([repr(float(v)) for v in p])


def adapt_S(S, ar, max_S):
    """Acceptance-driven change of the bisection level (pimc_utils.py:272-279)."""
    if ar > 0.5:
        S = min(max_S, S + 2)
    if 0.2 < ar < 0.5:
        S = min(max_S, S + 1)
    if ar < 0.1:
        S = max(1, S - 1)
    return S


def clamp_S(S, walkers_per_group, N, maxWGSize):
    minS = int(np.ceil(np.log2(walkers_per_group * N / float(maxWGSize))))
    maxS = int(np.log2(N))
    if maxS < minS:
        raise Exception('Too many walkers per workgroup')
    return min(maxS, max(minS, S))


def modN(ka, startXList, savePathsInterval, experimentName, opRunsFormula,
         mStepsPerOPRun, runsPerN, maxWGSize, continueRun=False, finalN=-1,
         simTime=-1, verbosity=0, cont_S=None, cont_N=None, cont_path=None,
         resultsDir="results", checkpointEvery=0, resumeCheckpoint=None, maxRuns=None):
    """Run the simulation with N doubling; see the module docstring.  ``maxRuns`` (new) stops
    after that many runs in total (handy for tests); ``resultsDir`` replaces "results"."""
    kaMod = copy.copy(ka)
    if kaMod.enableBisection is False:
        raise Exception('This function currently only works with bisection sampling')
    if continueRun:
        if cont_path is None:
            raise NameError('cont_path need to be defined if continueRun is enabled')
        if cont_S is None:
            raise NameError('cont_S need to be defined if continueRun is enabled')
        if cont_N is None:
            raise NameError('cont_N need to be defined if continueRun is enabled')
        kaMod.N = cont_N
        kaMod.S = cont_S
    else:
        kaMod.N = ka.N
        kaMod.S = 1
    startClock = time()
    pathChanges = 0
    timestamp = datetime.now().strftime("%Y-%m-%d/%H.%M.%S")
    outdir = os.path.join(resultsDir, experimentName, timestamp)
    os.makedirs(outdir, exist_ok=True)
    filename = os.path.join(outdir, "data")
    with open(os.path.join(outdir, "systemInfo"), "a"):
        pass

    ckpt = None
    if resumeCheckpoint is not None:
        with np.load(resumeCheckpoint) as z:
            ckpt = {k: z[k] for k in z.files}
        kaMod.N = int(ckpt["modn_N"])
        kaMod.S = int(ckpt["modn_S"])
        pathChanges = int(ckpt["modn_pathChanges"])

    firstNRun = True
    totRuns = 0 if ckpt is None else int(ckpt["modn_totRuns"])
    oldPaths = None
    while finalN == -1 or kaMod.N <= finalN:
        overheadClock = time()
        kaMod.S = clamp_S(kaMod.S, ka.nbrOfWalkersPerWorkGroup, kaMod.N, maxWGSize)
        kaMod.operatorRuns = opRunsFormula(kaMod.N, kaMod.S)
        kaMod.metroStepsPerOperatorRun = mStepsPerOPRun(kaMod.N, kaMod.S)
        kernel = PIMCKernel(kaMod, verbose=verbosity >= 2)
        if verbosity > 0:
            print("New kernel compiled, getStats():")
            print(kernel.getStats())
            print("Run results:")
        if ka.enableRanlux:
            kernel.initRanlux()
            kernel._queue.finish()
            kernel.groupInitRanlux()
            kernel._queue.finish()

        nRuns = 1
        if ckpt is not None:
            kernel.restoreState({k: v for k, v in ckpt.items() if not k.startswith("modn_")})
            nRuns = int(ckpt["modn_nRuns"]) + 1
            ckpt = None
        elif firstNRun:
            if not continueRun:
                initialPaths = straight_paths(startXList, ka.nbrOfWalkers, kaMod.system.DOF, kaMod.N)
            else:
                initialPaths = read_paths_csv(cont_path, ka.nbrOfWalkers, kaMod.N * kaMod.system.DOF)
            kernel.setPaths(initialPaths)
        else:
            kernel.setPaths(interpolate_paths(oldPaths, kaMod.system.DOF, kaMod.N // 2))

        runsThisN = runsPerN(kaMod.N, kaMod.S)
        lastCall = time()
        loopClock = time()
        while nRuns <= runsThisN or kaMod.N == finalN:
            if simTime != -1 and simTime != 0 and time() - startClock > simTime:
                if verbosity > 0:
                    print("Time limit reached!")
                kernel.close()
                return
            if maxRuns is not None and totRuns >= maxRuns:
                kernel.close()
                return
            kernel.run()
            if totRuns > 100 and totRuns % 100 == 0:
                kernel._queue.finish()
            pathChanges += kernel.getMetroStepsPerRun()
            _output(filename, kaMod.N, time() - startClock, pathChanges,
                    kernel.getAcceptanceRate(), kernel.getOperators(),
                    (time() - lastCall), kernel.getRunTime(), ka.beta, kaMod.S,
                    verbose=verbosity > 0)
            lastCall = time()
            if nRuns % savePathsInterval == 0 or nRuns == runsThisN:
                write_paths_csv(os.path.join(outdir, "pathsN" + str(kaMod.N) + "episode"
                                             + str(int(nRuns / savePathsInterval))), kernel.getPaths())
                if verbosity > 0:
                    print("Paths saved!")
            if checkpointEvery and nRuns % checkpointEvery == 0:
                st = kernel.getState()
                st.update(modn_N=np.array(kaMod.N), modn_S=np.array(kaMod.S),
                          modn_nRuns=np.array(nRuns), modn_totRuns=np.array(totRuns + 1),
                          modn_pathChanges=np.array(pathChanges))
                tmp = os.path.join(outdir, "checkpoint.tmp.npz")
                np.savez(tmp, **st)
                os.replace(tmp, os.path.join(outdir, "checkpoint.npz"))
            if simTime == 0 and nRuns == runsThisN and kaMod.N == finalN:
                if verbosity > 0:
                    print("Runs completed!")
                kernel.close()
                return
            nRuns += 1
            totRuns += 1
        loopClockEnd = time()
        with open(os.path.join(outdir, "timestamps"), "a") as f2:
            f2.write('N: ' + str(kaMod.N) + '\tS: ' + str(kaMod.S) + '\ttotRuns: ' + str(totRuns)
                     + '\ttime: ' + str(time() - startClock) + '\tnormtime: '
                     + str(float(time() - startClock) / (float(kernel._nbrOfThreads) * float(max(totRuns, 1))))
                     + '\n')
        if kaMod.N != finalN:
            oldPaths = kernel.getPaths()
            firstNRun = False
            ar = kernel.getAcceptanceRate()
            kaMod.S = adapt_S(kaMod.S, ar, int(np.log2(2 * kaMod.N)))
            kaMod.N *= 2
        kernel.close()
        if verbosity > 0:
            print('Overhead time: ' + str(time() - overheadClock + loopClock - loopClockEnd))


def _output(filename, N, t, pathChanges, acceptanceRate, operatorMean, hostRunTime,
            kernelRunTime, beta, S, verbose=False):
    """Append one run to <filename>.tsv (pimc_utils.py:287-355)."""
    if verbose:
        print("N: " + str(N) + "\tS: " + str(S) + "\tbeta: " + str(beta) + "\tAR: "
              + str(acceptanceRate) + "\tOPs: " + str(np.mean(operatorMean, axis=1))
              + "\tTime: [" + str(hostRunTime) + "," + str(kernelRunTime) + "]")
    path = filename + ".tsv"
    new = not os.path.exists(path) or os.path.getsize(path) == 0
    with open(path, "a") as f:
        if new:
            f.write("#Beta: " + str(beta) + "\n")
            f.write("#N\tTime\tpathChanges\tAR\tS")
            for i in range(len(operatorMean)):
                for j in range(len(operatorMean[0])):
                    f.write("\tOperator " + str(i) + ", Walker " + str(j))
            f.write("\n")
        f.write(str(N) + "\t" + str(t) + "\t" + str(pathChanges) + "\t" + str(acceptanceRate)
                + "\t" + str(S) + "\t")
        for walkerOperators in operatorMean:
            for op in walkerOperators:
                f.write(str(op) + "\t")
        f.write("\n")


def read_tsv(filename):
    """Parse a modN data.tsv: (beta, rows of (N, time, pathChanges, AR, S), operator array
    (runs, nOps, walkers))."""
    beta, header, rows, ops = None, None, [], []
    with open(filename) as f:
        for line in f:
            if line.startswith("#Beta:"):
                beta = float(line.split(":", 1)[1])
                continue
            if line.startswith("#"):
                header = line.rstrip("\n").split("\t")
                continue
            v = [x for x in line.rstrip("\n").split("\t") if x != ""]
            rows.append((int(v[0]), float(v[1]), int(v[2]), float(v[3]), int(v[4])))
            ops.append([float(x) for x in v[5:]])
    nops = len({h.split(",")[0] for h in header[5:]}) if header else 0
    arr = np.array(ops).reshape(len(ops), nops, -1) if nops else np.zeros((len(ops), 0, 0))
    return beta, rows, arr
