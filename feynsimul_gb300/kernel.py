"""PIMCKernel: the reference's kernel object (FeynSimul/kernel.py:47-801) on GB300.

Same constructor, methods, return shapes and exception types/messages as the reference,
so ``pimc_utils.modN``, the examples and user scripts run unchanged.  Behind it is the
C ABI of libfeynsimul_gb300.so (include/feynsimul.h): NVRTC specialises the sm_103a sweep
kernel for the plugin's strings and the run parameters, and all device buffers stay
resident between calls.  There is no CPU path: without the shared object (or a GPU) the
constructor raises.
"""
from __future__ import annotations

import copy
import ctypes

import numpy as np

from . import _lib
from ._lib import FsConfig, FsInfo, check, lib, strings

_ACCUM = {"fp32": _lib.ACCUM_REF_FP32, "fp64": _lib.ACCUM_FP64, "kahan": _lib.ACCUM_KAHAN,
          "study": _lib.ACCUM_STUDY}
_PARTIALS = {"fp32": _lib.FS_PARTIALS_FP32, "exact": _lib.FS_PARTIALS_EXACT}


def humanReadableSize(size):
    """Size in bytes in human readable form (kernel.py:28-42)."""
    if size <= 0 or size >= 10e18:
        return "%.3g" % size + " B"
    p = int(np.log(size) / np.log(1024))
    names = ["", "ki", "Mi", "Gi", "Ti", "Pi", "Ei"]
    return "%.3g" % (size / 1024.0 ** p) + " " + names[p] + "B"


class _Queue:
    """Stand-in for the OpenCL command queue: ``kernel._queue.finish()`` (pimc_utils.py:187)."""

    def __init__(self, k):
        self._k = k

    def finish(self):
        self._k.sync()


class PIMCKernel:
    """Builds the sweep for one KernelArgs and keeps its buffers on the GPU."""

    def __init__(self, ka, verbose=False):
        self._handle = None
        self._enableBins = ka.enableBins
        self._enableOperator = ka.enableOperator
        self._enableCorrelator = ka.enableCorrelator
        self._enablePathShift = ka.enablePathShift
        self._enableBisection = ka.enableBisection
        self._enableSingleNodeMove = ka.enableSingleNodeMove
        self._enableParallelizePath = ka.enableParallelizePath
        self._enableGlobalPath = ka.enableGlobalPath
        self._enableGlobalOldPath = ka.enableGlobalOldPath
        self._enableDouble = bool(ka.enableDouble)
        self._nbrOfWalkers = ka.nbrOfWalkers
        self._nbrOfWalkersPerWorkGroup = ka.nbrOfWalkersPerWorkGroup
        self._enableRanlux = bool(ka.enableRanlux)
        self._luxuaryFactor = ka.luxuaryFactor
        self._ranluxIntMax = ka.ranluxIntMax
        self._N = ka.N
        self._S = ka.S
        self._beta = ka.beta
        self._operatorRuns = ka.operatorRuns
        self._metroStepsPerOperatorRun = ka.metroStepsPerOperatorRun
        self._system = copy.copy(ka.system)
        self._compat = bool(getattr(ka, "compat", False))
        self._accumulation = getattr(ka, "accumulation", "fp64") or "fp64"
        self._partials = getattr(ka, "partials", "fp32") or "fp32"
        self._fastMath = bool(getattr(ka, "fastMath", True))
        self._walkersPerBlock = int(getattr(ka, "walkersPerBlock", 0) or 0)
        self._seed = getattr(ka, "seed", None)
        self._operators = ()
        self._correlators = ()
        self._runsSinceZero = 0
        self._kernelTime = None

        # ---- parameter checks, kernel.py:93-211 (same exception types and messages) ----
        if not isinstance(self._beta, float):
            raise TypeError('beta need to be a float')
        if self._enableOperator:
            self._operators = ka.operators
            if self._operatorRuns is None:
                raise NameError('operatorRuns need to be set if enableOperator is True.')
            if self._operators is None:
                raise NameError('operators need to be set if enableOperator is True.')
            if self._metroStepsPerOperatorRun is None:
                raise NameError('metroStepsPerOperatorRun need to be set if enableOperator is True.')
            if not isinstance(self._operators, tuple):
                raise TypeError('operators need to be a tuple of strings.')
        if self._enableCorrelator:
            self._correlators = ka.correlators
            if self._correlators is None:
                raise NameError('correlators need to be set if enableCorrelator is True.')
            if not isinstance(self._correlators, tuple):
                raise TypeError('correlators need to be a tuple of strings.')
        if self._enableSingleNodeMove:
            if ka.alpha is None:
                raise NameError('alpha need to be set if enableSingleNodeMove is True.')
        if self._enablePathShift:
            if ka.PSAlpha is None:
                raise NameError('PSALpha need to be set if enablePathShift is True')
        if self._enableRanlux:
            if self._luxuaryFactor is None or self._luxuaryFactor < 0:
                raise NameError('luxuaryFactor needs to be an uint >= 0.')
            if not isinstance(self._luxuaryFactor, (int, np.integer)):
                raise NameError('luxuaryFactor needs to be an integer.')
            if self._ranluxIntMax is None or self._ranluxIntMax <= 0:
                raise NameError('ranluxIntMax needs to be an uint > 0.')
            if not isinstance(self._ranluxIntMax, (int, np.integer)):
                raise NameError('ranluxIntMax needs to be an integer.')
        if self._enableBins:
            self._binResolutionPerDOF = ka.binResolutionPerDOF
            self._xMin = ka.xMin
            self._xMax = ka.xMax
            if self._xMin is None:
                raise NameError('xMin need to be set if enableBins is True.')
            if self._xMax is None:
                raise NameError('xMax need to be set if enableBins is True.')
            if self._binResolutionPerDOF is None:
                raise NameError('binResolutionPerDOF need to be set if enableBins is True.')
        if self._nbrOfWalkers % self._nbrOfWalkersPerWorkGroup != 0:
            raise Exception("The number of walkers must be a multiple "
                            "of the number of walkers per work group.")
        if self._nbrOfWalkers < self._nbrOfWalkersPerWorkGroup:
            raise Exception("The number of walkers per group must be less "
                            "than or equal to the total number of walkers")
        if not (self._N != 0 and ((self._N & (self._N - 1)) == 0)):
            raise Exception("Path node number, N, must be a power of 2.")
        if self._enableBisection:
            if self._S is None:
                raise NameError('S need to be set if enableBisection is True')
            if 2 ** self._S > self._N:
                raise Exception("2^S must be less than or equal to N.")
            if self._enableGlobalPath is None:
                raise NameError('enableGlobalPath need to be set if enableBisection is True.')
            if self._enableGlobalOldPath is None:
                raise NameError('enableGlobalOldPath need to be set if enableBisection is True.')
            if self._enableParallelizePath is None:
                raise NameError('enableParallelizePath need to be set if enableBisection is True')
        if self._enableParallelizePath:
            if self._enableSingleNodeMove:
                raise Exception("Single node move not possible when enableParallelizePath is True.")
            if self._enablePathShift:
                raise Exception("Shift path not possible when enableParallelizePath is True.")
        if self._enableGlobalOldPath and not self._enableBisection:
            raise Exception("Old Path is not used when bisection is not enabled")
        if not (self._enableBisection or self._enableSingleNodeMove or self._enablePathShift):
            raise Exception("at least one of enableBisection, enablePathShift and enableSingleNodeMove "
                            "must be True")
        if self._operatorRuns is None:
            raise NameError('operatorRuns need to be set.')
        if self._metroStepsPerOperatorRun is None:
            raise NameError('metroStepsPerOperatorRun need to be set.')
        if self._accumulation not in _ACCUM:
            raise ValueError("accumulation must be one of " + ", ".join(_ACCUM))
        if self._partials not in _PARTIALS:
            raise ValueError("partials must be one of " + ", ".join(_PARTIALS))

        if self._enableParallelizePath:
            self._threadsPerWalker = self._N // (2 ** self._S)
        else:
            self._threadsPerWalker = 1
        self._nbrOfThreads = self._nbrOfWalkers * self._threadsPerWalker
        self._nbrOfWorkgroups = self._nbrOfWalkers // self._nbrOfWalkersPerWorkGroup

        hists = tuple(getattr(ka, "histograms", None) or ())
        hbins = int(getattr(ka, "histBins", None) or 0)
        hrange = getattr(ka, "histRange", None) or (0.0, 1.0)
        self._histograms, self._histBins, self._histRange = hists, (hbins if hists else 0), hrange

        c = FsConfig()
        c.dof = self._system.DOF
        c.n_slices = self._N
        c.bisection_level = self._S if self._S is not None else 1
        c.beta = self._beta
        c.n_walkers = self._nbrOfWalkers
        c.walkers_per_group = self._nbrOfWalkersPerWorkGroup if self._enableParallelizePath else 1
        c.operator_runs = self._operatorRuns
        c.metro_steps_per_operator_run = self._metroStepsPerOperatorRun
        c.enable_parallelize_path = int(bool(self._enableParallelizePath))
        c.enable_ranlux = int(self._enableRanlux)
        c.luxury_factor = int(self._luxuaryFactor or 0)
        c.ranlux_int_max = int(self._ranluxIntMax or 1)
        c.enable_double = int(self._enableDouble)
        c.enable_bins = int(bool(self._enableBins))
        if self._enableBins:
            c.x_min, c.x_max, c.bin_resolution_per_dof = float(self._xMin), float(self._xMax), int(self._binResolutionPerDOF)
        c.hist_lo, c.hist_hi = float(hrange[0]), float(hrange[1])
        c.hist_bins = self._histBins
        c.compat = int(self._compat)
        c.accum = _ACCUM[self._accumulation]
        c.partials = _PARTIALS[self._partials]
        c.fast_math = int(self._fastMath)
        c.walkers_per_block = self._walkersPerBlock
        c.min_blocks_per_sm = int(getattr(ka, "minBlocksPerSM", 0) or 0)
        c.learned = int(bool(getattr(ka, "learnedProposal", False)))
        # enableGlobalOldPath (kernel.c:259-276) has no counterpart: the saved old segment
        # is per-thread private data either way (registers, spilling to local memory)
        c.global_path = int(bool(self._enableGlobalPath)) if self._enableBisection else 0
        pc = getattr(ka, "potentialCache", None)
        if not (pc is None or isinstance(pc, bool) or pc == "device"):
            raise ValueError("potentialCache must be None, True, False or 'device'")
        c.potential_cache = 0 if pc is None else (3 if pc == "device" else (1 if pc else 2))
        c.moves = ((_lib.FS_MOVE_BISECTION if self._enableBisection else 0)
                   | (_lib.FS_MOVE_PATH_SHIFT if self._enablePathShift else 0)
                   | (_lib.FS_MOVE_SINGLE_NODE if self._enableSingleNodeMove else 0))
        c.alpha = float(ka.alpha) if self._enableSingleNodeMove else 0.0
        c.ps_alpha = float(getattr(ka, "PSAlpha", None) or 0.0) if self._enablePathShift else 0.0
        self._movesPerStep = bin(c.moves).count("1")
        self._learned = bool(c.learned)
        self._cfg = c

        L = lib()
        ops, nops = strings(self._operators)
        cors, ncor = strings(self._correlators)
        hs, nh = strings(hists)
        h = ctypes.c_void_p()
        rc = L.fs_create(ctypes.byref(c), self._system.potential.encode(),
                         (getattr(self._system, "userCode", "") or "").encode(),
                         ops, nops, cors, ncor, hs, nh, ctypes.byref(h))
        if rc == _lib.FS_ERR_OOM:
            raise Exception("Unable to allocate global memory on device, out of memory?")
        check(rc, None)
        self._handle = h
        self._queue = _Queue(self)
        info = FsInfo()
        check(L.fs_query(h, ctypes.byref(info)), h)
        self._info = info
        if verbose:
            with open("cleaned.cu", "w") as f:
                f.write(self.getSource())
            print("Saved the generated CUDA source in cleaned.cu")

        # ---- seed tables, drawn like kernel.py:396-426 ----
        rs = np.random if self._seed is None else np.random.RandomState(self._seed)
        if self._enableRanlux:
            self._seeds = rs.randint(0, high=2 ** 31 - 1, size=(self._nbrOfThreads + 1)).astype(np.uint32)
            self._groupSeeds = rs.randint(0, high=2 ** 31 - 1,
                                          size=(self._N // (2 ** self._S) + 1)).astype(np.uint32)
        else:
            self._seeds = rs.randint(0, high=2 ** 31 - 1, size=(self._nbrOfThreads + 1, 4)).astype(np.uint32)
            check(L.fs_set_xorshift_seeds(h, self._seeds.ctypes.data, self._seeds.shape[0]), h)
            if not self._compat:
                self._walkerSeeds = rs.randint(0, high=2 ** 31 - 1,
                                               size=(self._nbrOfWalkers, 4)).astype(np.uint32)
                check(L.fs_set_walker_seeds(h, self._walkerSeeds.ctypes.data, self._nbrOfWalkers), h)
            self._ranlux_ready = True
        self._ranlux_ready = not self._enableRanlux

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if self._handle is not None:
            lib().fs_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(lib().fs_sync(self._handle), self._handle)

    # ------------------------------------------------------------------ run
    def run(self, launches=1, wait=True):
        """One reference run() (operatorRuns x metroStepsPerOperatorRun sweeps), kernel.py:459-506.

        ``launches`` > 1 queues several runs back to back; ``wait=False`` returns at once
        (the queue is then drained by ``_queue.finish()`` or any getter)."""
        check(lib().fs_run(self._handle, int(launches)), self._handle)
        self._runsSinceZero += int(launches)
        if wait:
            self.sync()

    def runHost(self, paths, out=None, launches=1, chunks=0):
        """setPaths(paths) + run(launches) + getPaths(out) as one pipelined call: the walkers
        are split into ``chunks`` chunks (0: automatic from the grid and the occupancy) whose
        host-to-device copy, sweeps and copy back overlap (fs_run_host).  Same results bit for bit.  The copies overlap only when
        ``paths`` and ``out`` are page-locked (``pinHost``).  Returns ``out``."""
        a = np.asarray(paths)
        n = self._nbrOfWalkers * self._N * self._system.DOF
        if a.dtype != self._ftype or not a.flags["C_CONTIGUOUS"] or a.size != n:
            raise ValueError("paths must be a C-contiguous array of the paths' size and dtype")
        if out is None:
            out = np.empty((self._nbrOfWalkers, self._N * self._system.DOF), self._ftype)
        elif out.dtype != self._ftype or not out.flags["C_CONTIGUOUS"] or out.size != n:
            raise ValueError("out must be a C-contiguous array of the paths' size and dtype")
        check(lib().fs_run_host(self._handle, a.ctypes.data, out.ctypes.data, int(launches), int(chunks)),
              self._handle)
        used = ctypes.c_int32()
        check(lib().fs_get_last_chunks(self._handle, ctypes.byref(used)), self._handle)
        self.lastChunks = int(used.value)
        self._runsSinceZero += int(launches)
        self.sync()
        return out

    @staticmethod
    def pinHost(array):
        """Page-lock a numpy array's memory for overlapped copies (undo with unpinHost)."""
        check(lib().fs_pin_host(array.ctypes.data, array.nbytes))

    @staticmethod
    def unpinHost(array):
        check(lib().fs_unpin_host(array.ctypes.data))

    def _thread_rows_compat_group(self):
        """Group-seed index of every thread: group + lid1 * nWG (kernel.c:165)."""
        T, WPG, nWG = self._threadsPerWalker, self._nbrOfWalkersPerWorkGroup, self._nbrOfWorkgroups
        w = np.repeat(np.arange(self._nbrOfWalkers), T)
        t = np.tile(np.arange(T), self._nbrOfWalkers)
        if self._enableParallelizePath:
            g, l1 = w // WPG, w % WPG
            tid = g * T + t + l1 * nWG * T
            idx = g + l1 * nWG
        else:
            tid, idx = w, w
        rows = np.empty(self._nbrOfThreads, np.int64)
        rows[tid] = idx
        return rows

    def initRanlux(self):
        """Seed the per-thread RANLUX table (kernel.py:508-530).

        Reference-compatible mode seeds every row from seeds[0] (kernel.c:155); otherwise
        row i gets the unique value (seeds[0] << 32) + i."""
        if not self._enableRanlux:
            raise Exception("RANLUX is not enabled")
        base = int(self._seeds[0])
        if self._compat:
            xs = np.full(self._nbrOfThreads, base, np.uint64)
        else:
            xs = (np.uint64(base) << np.uint64(32)) + np.arange(self._nbrOfThreads, dtype=np.uint64)
        check(lib().fs_ranlux_init(self._handle, xs.ctypes.data, xs.shape[0]), self._handle)

    def groupInitRanlux(self):
        """Seed the walker-offset RANLUX streams (kernel.py:532-554)."""
        if not self._enableRanlux:
            raise Exception("RANLUX is not enabled")
        if self._compat:
            rows = self._thread_rows_compat_group()
            if rows.max() >= self._groupSeeds.shape[0]:
                raise Exception("the reference reads groupSeeds out of bounds for this many walkers "
                                "(kernel.py:417-420 vs kernel.c:165); use compat=False")
            xs = self._groupSeeds[rows].astype(np.uint64)
        else:
            base = (int(self._seeds[0]) ^ 0x80000000) << 32
            xs = np.uint64(base) + np.arange(self._nbrOfWalkers, dtype=np.uint64)
        check(lib().fs_ranlux_group_init(self._handle, xs.ctypes.data, xs.shape[0]), self._handle)
        self._ranlux_ready = True

    # ------------------------------------------------------------------ data
    @property
    def _ftype(self):
        return np.float64 if self._enableDouble else np.float32

    def getPaths(self, out=None):
        """Paths, shape (walkers, N * DOF), DOF-major per walker (kernel.py:557-565).
        ``out`` may be a preallocated C-contiguous array of that shape and dtype."""
        if out is None:
            out = np.empty((self._nbrOfWalkers, self._N * self._system.DOF), self._ftype)
        elif out.dtype != self._ftype or not out.flags["C_CONTIGUOUS"] or \
                out.size != self._nbrOfWalkers * self._N * self._system.DOF:
            raise ValueError("out must be a C-contiguous array of the paths' shape and dtype")
        check(lib().fs_get_paths(self._handle, out.ctypes.data, out.size), self._handle)
        return out

    def setPathsTiled(self, template):
        """Fill every walker's path from a few template walkers (shape (k, N * DOF)):
        walker w gets template w % k, replicated on the device."""
        a = np.ascontiguousarray(np.asarray(template), dtype=self._ftype)
        per = self._N * self._system.DOF
        if a.size % per or a.size == 0:
            raise ValueError("template must hold whole walkers of N * DOF elements")
        check(lib().fs_set_paths_tiled(self._handle, a.ctypes.data, a.size // per), self._handle)

    def setPaths(self, paths):
        """Set the paths (kernel.py:567-574)."""
        a = np.ascontiguousarray(np.asarray(paths), dtype=self._ftype)
        if a.size != self._nbrOfWalkers * self._N * self._system.DOF:
            raise ValueError("paths must have nbrOfWalkers * N * DOF elements")
        check(lib().fs_set_paths(self._handle, a.ctypes.data, a.size), self._handle)

    def _raw_operators(self):
        n = self._nbrOfThreads * len(self._operators) * (3 if self._accumulation == "study" else 1)
        out = np.empty(n, np.float64)
        check(lib().fs_get_operators(self._handle, out.ctypes.data, n), self._handle)
        return out

    def getOperators(self):
        """Per-walker operator means, shape (nOps, walkers) (kernel.py:576-606).

        In reference-compatible mode the reduction repeats the reference's index arithmetic
        exactly (which mixes walkers when nbrOfWalkersPerWorkGroup > 1); otherwise each
        walker's own work-items are averaged.  In "study" accumulation the FP64 column is
        returned (see getOperatorsStudy for all three)."""
        if not self._enableOperator:
            raise Exception("Can only return operator when created with"
                            "kernelArg.enableOperator = True")
        nops = len(self._operators)
        if not self._compat and self._accumulation != "study":
            # the walkers' own thread means, averaged on the device
            out = np.empty((nops, self._nbrOfWalkers), np.float64)
            check(lib().fs_get_walker_operators(self._handle, out.ctypes.data, out.size), self._handle)
            return out
        raw = self._raw_operators()
        if self._accumulation == "study":
            raw = raw.reshape(-1, 3)[:, 2]
        T = self._threadsPerWalker
        if self._compat or not self._enableParallelizePath:
            per = raw.reshape(-1)
            if self._enableParallelizePath:
                idx = (np.arange(self._nbrOfWalkers)[:, None] * nops * T + np.arange(T)[None, :] * nops)
                return np.stack([per[j + idx].mean(axis=1) for j in range(nops)])
            return per.reshape(self._nbrOfWalkers, nops).T.copy()
        return self._per_walker(raw.reshape(self._nbrOfThreads, nops)).T.copy()

    def _per_walker(self, per_thread):
        """(threads, k) in reference thread-id order -> (walkers, k) means over each walker's threads."""
        T, WPG, nWG = self._threadsPerWalker, self._nbrOfWalkersPerWorkGroup, self._nbrOfWorkgroups
        w = np.arange(self._nbrOfWalkers)
        g, l1 = w // WPG, w % WPG
        tid = (g * T + l1 * nWG * T)[:, None] + np.arange(T)[None, :]
        return per_thread[tid].mean(axis=1)

    def getOperatorsStudy(self):
        """Precision study: (3, nOps, walkers) means from FP32, Kahan-FP32 and FP64 sums."""
        if self._accumulation != "study":
            raise Exception("create the kernel with accumulation='study'")
        nops = len(self._operators)
        raw = self._raw_operators().reshape(self._nbrOfThreads, nops, 3)
        return np.stack([self._per_walker(raw[:, :, k]).T for k in range(3)])

    def getCorrelator(self):
        """(mean (nCorr, N/2), standard error) (kernel.py:608-617).

        The device keeps running sums.  The reference divides by one run's count however many
        runs were made (its buffer is never re-zeroed); reference-compatible mode repeats
        that, otherwise the sums are divided by the runs made since creation or
        zeroAccumulators().

        The standard error is that of the mean: the per-walker spread / sqrt(walkers) of the
        same normalised values.  The reference leaves its standard error in raw-sum units,
        operatorRuns * N times the mean's scale (kernel.py:613-616); reference-compatible
        mode repeats that."""
        if not self._enableCorrelator:
            raise Exception("Can only return correlator when created with"
                            "kernalArg.enableCorrelator = True")
        raw = self._raw_correlator()
        if self._accumulation == "study":
            raw = raw.reshape(-1, 4)[:, 3]
        vals = raw.reshape(self._nbrOfWalkers, len(self._correlators), self._N // 2)
        runs = 1 if self._compat else max(1, self._runsSinceZero)
        vals = vals / float(runs)
        scale = float(self._operatorRuns * self._N)
        mean = vals.mean(axis=0) / scale
        se = vals.std(axis=0) / np.sqrt(self._nbrOfWalkers)
        if not self._compat:
            se = se / scale
        return (mean, se)

    def getCorrelatorPerWalker(self):
        """Each walker's correlator mean, shape (walkers, nCorr, N/2), with getCorrelator's
        normalisation (its mean over the walkers is getCorrelator's mean); the FP64 column
        in "study" accumulation.  Used to merge replicas and for batch errors."""
        if not self._enableCorrelator:
            raise Exception("Can only return correlator when created with"
                            "kernalArg.enableCorrelator = True")
        raw = self._raw_correlator()
        if self._accumulation == "study":
            raw = raw.reshape(-1, 4)[:, 3]
        return raw.reshape(self._nbrOfWalkers, len(self._correlators), self._N // 2) * self._cor_norm()

    def getMovesPerRun(self):
        """Moves each work-item makes in one run: the steps times the move types per step
        (the denominator of the per-move acceptance rate)."""
        return self._operatorRuns * self._metroStepsPerOperatorRun * self._movesPerStep

    def _cor_count(self):
        return self._nbrOfWalkers * len(self._correlators) * (self._N // 2) * \
            (4 if self._accumulation == "study" else 1)

    def _raw_correlator(self):
        n = self._cor_count()
        raw = np.empty(n, np.float64)
        check(lib().fs_get_correlator(self._handle, raw.ctypes.data, n), self._handle)
        return raw

    def _cor_norm(self):
        runs = 1 if self._compat else max(1, self._runsSinceZero)
        return 1.0 / (float(runs) * self._operatorRuns * self._N)

    def getCorrelatorStudy(self):
        """Precision study: per-walker correlator means (3, walkers, nCorr, N/2) from the plain
        FP32, Kahan-FP32 and FP64 sums of the same products."""
        if self._accumulation != "study":
            raise Exception("create the kernel with accumulation='study'")
        raw = self._raw_correlator().reshape(self._nbrOfWalkers, len(self._correlators), self._N // 2, 4)
        return np.stack([raw[..., 0], raw[..., 1], raw[..., 3]]) * self._cor_norm()

    def getCorrelatorMoments(self, walkers=None):
        """Correlator mean and standard error over a walker range (default all), reduced on
        the device: (mean, se), each (nCorr, N/2), or (3, nCorr, N/2) in "study"
        accumulation (plain FP32, Kahan, FP64 sums)."""
        if not self._enableCorrelator:
            raise Exception("Can only return correlator when created with"
                            "kernalArg.enableCorrelator = True")
        w0, w1 = walkers if walkers is not None else (0, self._nbrOfWalkers)
        ncol = 3 if self._accumulation == "study" else 1
        n = len(self._correlators) * (self._N // 2) * ncol
        s, q = np.empty(n, np.float64), np.empty(n, np.float64)
        check(lib().fs_reduce_correlator(self._handle, int(w0), int(w1), s.ctypes.data, q.ctypes.data, n),
              self._handle)
        nw = float(w1 - w0)
        f = self._cor_norm()
        mean = s / nw
        var = np.maximum(q / nw - mean * mean, 0.0)
        shape = (len(self._correlators), self._N // 2, ncol)
        mean = np.moveaxis((mean * f).reshape(shape), -1, 0)
        se = np.moveaxis((np.sqrt(var / nw) * f).reshape(shape), -1, 0)
        return (mean[0], se[0]) if ncol == 1 else (mean, se)

    def zeroAccumulators(self):
        """Reset correlator sums, bins and histogram counts."""
        check(lib().fs_zero_accumulators(self._handle), self._handle)
        self._runsSinceZero = 0

    def getBinCounts(self):
        """Normalised probability density on the DOF hypercube (kernel.py:619-637)."""
        if not self._enableBins:
            raise Exception("Can only return bins when kernalArg.enableBins = True")
        n = self._binResolutionPerDOF ** self._system.DOF
        raw = np.empty(n, np.uint32)
        check(lib().fs_get_bins(self._handle, raw.ctypes.data, n), self._handle)
        runs = 1 if self._compat else max(1, self._runsSinceZero)
        totBinCount = self._nbrOfWalkers * self._operatorRuns * self._N * runs
        binVol = (float(self._xMax - self._xMin) / float(self._binResolutionPerDOF)) ** self._system.DOF
        shape = (self._binResolutionPerDOF,) * self._system.DOF
        return (raw.astype(self._ftype) / (binVol * totBinCount)).reshape(shape)

    def getBinCountsRaw(self):
        n = self._binResolutionPerDOF ** self._system.DOF
        raw = np.empty(n, np.uint32)
        check(lib().fs_get_bins(self._handle, raw.ctypes.data, n), self._handle)
        return raw

    def getHistogram(self, density=True):
        """Histogram of the ``histograms`` expressions: (bin centres, values).  With
        density=True the counts are normalised to a probability density per expression."""
        if not self._histBins:
            raise Exception("create the kernel with histograms and histBins")
        raw = np.empty(self._histBins, np.uint64)
        check(lib().fs_get_histogram(self._handle, raw.ctypes.data, self._histBins), self._handle)
        lo, hi = self._histRange
        w = (hi - lo) / self._histBins
        centres = lo + (np.arange(self._histBins) + 0.5) * w
        if not density:
            return centres, raw
        total = (self._nbrOfWalkers * self._operatorRuns * self._N * len(self._histograms)
                 * max(1, self._runsSinceZero))
        return centres, raw.astype(np.float64) / (total * w)

    def getRunTime(self):
        """Device time of the last run() call in seconds (kernel.py:638-646)."""
        t = ctypes.c_double()
        check(lib().fs_get_run_time(self._handle, ctypes.byref(t)), self._handle)
        return t.value

    def getAccepts(self):
        out = np.empty(self._nbrOfThreads, np.uint32)
        check(lib().fs_get_accepts(self._handle, out.ctypes.data, out.size), self._handle)
        return out

    def getAcceptanceRate(self):
        """Mean acceptance rate of the last run (kernel.py:648-658).  The reference divides
        every move type's accepts by the steps alone (so walker mode with several move
        types can exceed 1); reference-compatible mode repeats that, otherwise the rate is
        per move."""
        moves = 1 if self._compat else self._movesPerStep
        return (self.getAccepts() / float(self._operatorRuns * self._metroStepsPerOperatorRun * moves)).mean()

    def getSeeds(self):
        out = np.empty((self._nbrOfThreads + 1, 4), np.uint32)
        check(lib().fs_get_xorshift_seeds(self._handle, out.ctypes.data, out.shape[0]), self._handle)
        return out

    def setSeeds(self, seeds):
        a = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(self._nbrOfThreads + 1, 4)
        check(lib().fs_set_xorshift_seeds(self._handle, a.ctypes.data, a.shape[0]), self._handle)

    def getWalkerSeeds(self):
        out = np.empty((self._nbrOfWalkers, 4), np.uint32)
        check(lib().fs_get_walker_seeds(self._handle, out.ctypes.data, out.shape[0]), self._handle)
        return out

    def setWalkerSeeds(self, seeds):
        a = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(self._nbrOfWalkers, 4)
        check(lib().fs_set_walker_seeds(self._handle, a.ctypes.data, a.shape[0]), self._handle)

    def _group_rows(self):
        return self._nbrOfThreads if self._compat else self._nbrOfWalkers

    def getRanluxTables(self):
        t = np.empty((self._nbrOfThreads, 28), np.uint32)
        g = np.empty((self._group_rows(), 28), np.uint32)
        check(lib().fs_get_ranlux_tables(self._handle, t.ctypes.data, t.shape[0], g.ctypes.data, g.shape[0]),
              self._handle)
        return t, g

    def setRanluxTables(self, tab, group_tab):
        t = np.ascontiguousarray(tab, dtype=np.uint32).reshape(self._nbrOfThreads, 28)
        g = np.ascontiguousarray(group_tab, dtype=np.uint32).reshape(self._group_rows(), 28)
        check(lib().fs_set_ranlux_tables(self._handle, t.ctypes.data, t.shape[0], g.ctypes.data, g.shape[0]),
              self._handle)
        self._ranlux_ready = True

    # ------------------------------------------------------------------ learned proposal
    def setLearnedProposal(self, model):
        """Load a feynsimul_gb300.learned.LearnedProposal into the sweep (the kernel must be
        built with learnedProposal=True).  The model's sigma_1 must be this kernel's
        level-1 bisection width."""
        if not self._learned:
            raise Exception("create the kernel with learnedProposal=True")
        from .learned import sigma_level
        s1 = sigma_level(self._beta, self._N, self._S, 1)
        if abs(model.sigma1 - s1) > 1e-6 * s1:
            raise ValueError(f"model was trained for sigma_1 = {model.sigma1}, this kernel has {s1}")
        if model.dof != self._system.DOF:
            raise ValueError("model DOF differs from the system's")
        frag, bias = model.packed()
        check(lib().fs_set_learned_proposal(self._handle, frag.ctypes.data, frag.nbytes, bias.ctypes.data,
                                            bias.size, 1.0 / model.length_scale), self._handle)
        self._model = model

    # ------------------------------------------------------------------ checkpoints
    def _config_fingerprint(self):
        c = self._cfg
        fields = {name: getattr(c, name) for name, _ in c._fields_}
        strs = (self._system.potential, getattr(self._system, "userCode", ""), self._operators,
                self._correlators, self._histograms)
        return repr((sorted(fields.items()), strs))

    def getState(self):
        """Everything a continuation needs, as numpy arrays: paths, RNG tables, running sums,
        and the run counter.  restoreState() on a kernel built from the same KernelArgs
        continues bit for bit as if the run had not stopped."""
        L = lib()
        steps = ctypes.c_uint64()
        check(L.fs_get_step_counter(self._handle, ctypes.byref(steps)), self._handle)
        st = {"paths": self.getPaths(), "runs_since_zero": np.array(self._runsSinceZero),
              "fingerprint": np.array(self._config_fingerprint()), "step_counter": np.array(steps.value, np.uint64)}
        if self._enableRanlux:
            st["ranlux_tab"], st["group_tab"] = self.getRanluxTables()
        else:
            st["seeds"] = self.getSeeds()
            if not self._compat:
                st["walker_seeds"] = self.getWalkerSeeds()
        if self._enableCorrelator:
            st["correlator"] = self._raw_correlator()
        if self._enableBins:
            st["bins"] = self.getBinCountsRaw()
        if self._histBins:
            h = np.empty(self._histBins, np.uint64)
            check(L.fs_get_histogram(self._handle, h.ctypes.data, self._histBins), self._handle)
            st["histogram"] = h
        return st

    def restoreState(self, st):
        if str(st["fingerprint"]) != self._config_fingerprint():
            raise ValueError("checkpoint was written by a kernel with a different configuration")
        L = lib()
        self.setPaths(st["paths"])
        if self._enableRanlux:
            self.setRanluxTables(st["ranlux_tab"], st["group_tab"])
        else:
            self.setSeeds(st["seeds"])
            if not self._compat:
                self.setWalkerSeeds(st["walker_seeds"])
        if "correlator" in st:
            c = np.ascontiguousarray(st["correlator"], dtype=np.float64)
            check(L.fs_set_correlator(self._handle, c.ctypes.data, c.size), self._handle)
        if "bins" in st:
            b = np.ascontiguousarray(st["bins"], dtype=np.uint32)
            check(L.fs_set_bins(self._handle, b.ctypes.data, b.size), self._handle)
        if "histogram" in st:
            h = np.ascontiguousarray(st["histogram"], dtype=np.uint64)
            check(L.fs_set_histogram(self._handle, h.ctypes.data, h.size), self._handle)
        self._runsSinceZero = int(st["runs_since_zero"])
        if "step_counter" in st:
            check(L.fs_set_step_counter(self._handle, int(st["step_counter"])), self._handle)

    def saveCheckpoint(self, filename):
        np.savez(filename, **self.getState())

    def loadCheckpoint(self, filename):
        with np.load(filename) as z:
            self.restoreState({k: z[k] for k in z.files})

    # ------------------------------------------------------------------ info
    def getGlobalMemory(self):
        """Device memory held by this kernel, bytes (kernel.py:660-684)."""
        return int(self._info.device_bytes)

    def getStats(self):
        """Human readable resource usage (kernel.py:686-730)."""
        i = self._info
        return ("Global memory (used): " + humanReadableSize(self.getGlobalMemory()) + "\n"
                + "Shared memory per block (used/max): " + humanReadableSize(i.smem_bytes) + " / 227 kiB\n"
                + "Registers per thread: " + str(i.registers) + "\n"
                + "Block (walkers x threads per walker): (%d x %d) = %d threads\n"
                % (i.walkers_per_block, i.threads_per_walker, i.block_threads)
                + "Number of blocks (used): " + str(i.grid_blocks))

    def exceedsLimits(self):
        """False once the kernel exists: fs_create rejects configurations that do not fit."""
        return False

    def getBuildLog(self):
        return lib().fs_build_log(self._handle).decode(errors="replace")

    def getSource(self):
        return lib().fs_source(self._handle).decode(errors="replace")

    def getInfo(self):
        return self._info

    def getMetroStepsPerRun(self):
        """Metropolis steps in one run (kernel.py:787-801)."""
        if self._enableParallelizePath:
            return (self._nbrOfWalkers * self._threadsPerWalker * self._metroStepsPerOperatorRun
                    * self._operatorRuns * self._enableBisection)
        return (self._nbrOfWalkers * self._metroStepsPerOperatorRun * self._operatorRuns
                * (self._enableBisection + self._enablePathShift + self._enableSingleNodeMove))

    def getNodeUpdatesPerRun(self):
        """Interior time slices resampled per run: Metropolis steps x (2^S - 1)."""
        return self.getMetroStepsPerRun() * (2 ** self._S - 1)
