"""The reference's helium-cluster plugin under its module and class name
(FeynSimul/physical_systems/lm2m2_cluster.py:6-95): ``Lm2m2_cluster(n, T, ...)``.

The system is feynsimul_gb300.physical_systems.lm2m2.Lm2m2Cluster: mass-scaled Jacobi
coordinates, Angstrom and Kelvin, beta = 1 / T.  The reference builds its code with sympy;
``simplify``, ``verbose`` and ``enableDouble`` only steer that generation there and are
accepted here for the same calls (the kernel's precision follows KernelArgs.enableDouble).
"""
from .lm2m2 import GROUND_STATES, Lm2m2Cluster, reference_helper_code


class Lm2m2_cluster(Lm2m2Cluster):
    def __init__(self, n, T, useJacobi=True, simplify=True, verbose=False, enableDouble=False,
                 referenceDerivative=False):
        if not useJacobi:
            # the reference has no absolute-coordinate form either (lm2m2_cluster.py:12-14)
            raise Exception("disablement of jacobi isn't implemented yet")
        super().__init__(n, T, referenceDerivative=referenceDerivative)
        if 3 <= n <= 10:
            # the reference stores the magnitude (lm2m2_cluster.py:17-19)
            self.groundStateEnergy = GROUND_STATES[n - 3]
        # the reference's helper names (sqr, lm2m2sqrt, dlm2m2sqrtdr) for user operators
        self.userCode += reference_helper_code()
