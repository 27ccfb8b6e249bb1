"""KernelArgs: the run-parameter bag of the reference (FeynSimul/kernel_args.py:21-217).

Same constructor signature and attribute names, so reference scripts work unchanged.
Keyword-only additions of this engine:

* ``compat`` (False): reference-compatible random-number use -- per-thread xorshift rows
  with the walker's integer stream aliased to a seed row and never written back
  (kernel.c:568-572), RANLUX tables all seeded from ``seeds[0]`` (kernel.c:155) and
  RANLUX integers whose low bits are zero (kernel.c:206).  The default fixes these.
* ``accumulation`` ("fp64"): operator / correlator running sums: "fp64", "fp32" (the
  reference's FP32 sums in its order), "kahan" (compensated FP32) or "study" (all three
  side by side, for the precision study).
* ``partials`` ("fp32"): how one measurement's values are summed before their FP64 add to
  the running sums (FP32 builds, "fp64" accumulation; the correlator also in "kahan"):
  "fp32" (a thread's operator values over its slices in FP32, within gamma(2^S) of the
  exact sum; a lag's products in four fused multiply-add chains, within
  gamma(N/4 + 2) * C(0)) or "exact" (operator values added in FP64 one by one; the rounded
  products in float-float, about 48 bits).  The "study" accumulation uses "exact".
* ``fastMath`` (True): fast transcendental intrinsics, as the reference's
  ``-cl-fast-relaxed-math`` build; False gives IEEE functions and no FMA contraction.
* ``histograms`` / ``histRange`` / ``histBins``: plugin expressions binned into one shared
  histogram (e.g. the pair distances of a cluster).
* ``walkersPerBlock`` (0 = automatic): walkers per CUDA thread block.
* ``minBlocksPerSM`` (0 = as many as shared memory admits): thread blocks per SM the
  sweep kernel is compiled to fit, i.e. its register budget.
* ``learnedProposal`` (False): draw each segment's level-1 midpoint from a learned Gaussian
  (feynsimul_gb300.learned), Metropolis-Hastings corrected; load the model with
  PIMCKernel.setLearnedProposal.
* ``potentialCache`` (None = automatic): keep V of every slice between moves so a move
  evaluates the potential only at its proposed nodes (bit-identical results): True = in
  shared memory (costs occupancy), "device" = in device memory (N values per walker, L1/L2
  resident), False = off.
* ``seed`` (None): master seed for the seed tables; None draws from ``np.random`` exactly
  as kernel.py:412-426 does.
"""


class KernelArgs:

    def __init__(self,
                 system,
                 nbrOfWalkers,
                 N,
                 beta,
                 enableOperator,
                 enableCorrelator,
                 enableBisection,
                 enablePathShift,
                 enableSingleNodeMove,
                 enableBins,
                 nbrOfWalkersPerWorkGroup,
                 enableDouble=None,
                 enableRanlux=None,
                 luxuaryFactor=None,
                 ranluxIntMax=None,
                 S=None,
                 alpha=None,
                 PSAlpha=None,
                 enableParallelizePath=None,
                 metroStepsPerOperatorRun=None,
                 enableGlobalPath=None,
                 enableGlobalOldPath=None,
                 operators=None,
                 operatorRuns=None,
                 correlators=None,
                 xMin=None,
                 xMax=None,
                 binResolutionPerDOF=None,
                 *,
                 compat=False,
                 accumulation="fp64",
                 partials="fp32",
                 fastMath=True,
                 histograms=None,
                 histRange=None,
                 histBins=None,
                 walkersPerBlock=0,
                 minBlocksPerSM=0,
                 learnedProposal=False,
                 potentialCache=None,
                 seed=None):
        self.system = system
        self.nbrOfWalkers = nbrOfWalkers
        self.N = N
        self.S = S
        self.beta = beta
        self.nbrOfWalkersPerWorkGroup = nbrOfWalkersPerWorkGroup
        self.enablePathShift = enablePathShift
        self.enableDouble = enableDouble
        self.enableSingleNodeMove = enableSingleNodeMove
        self.alpha = alpha
        self.PSAlpha = PSAlpha
        self.enableOperator = enableOperator
        self.enableRanlux = enableRanlux
        self.luxuaryFactor = luxuaryFactor
        self.ranluxIntMax = ranluxIntMax
        self.operatorRuns = operatorRuns
        self.operators = operators
        self.metroStepsPerOperatorRun = metroStepsPerOperatorRun
        self.enableCorrelator = enableCorrelator
        self.correlators = correlators
        self.enableBins = enableBins
        self.xMin = xMin
        self.xMax = xMax
        self.binResolutionPerDOF = binResolutionPerDOF
        self.enableBisection = enableBisection
        self.enableParallelizePath = enableParallelizePath
        self.enableGlobalPath = enableGlobalPath
        self.enableGlobalOldPath = enableGlobalOldPath
        # additions
        self.compat = compat
        self.accumulation = accumulation
        self.partials = partials
        self.fastMath = fastMath
        self.histograms = histograms
        self.histRange = histRange
        self.histBins = histBins
        self.walkersPerBlock = walkersPerBlock
        self.minBlocksPerSM = minBlocksPerSM
        self.learnedProposal = learnedProposal
        self.potentialCache = potentialCache
        self.seed = seed
