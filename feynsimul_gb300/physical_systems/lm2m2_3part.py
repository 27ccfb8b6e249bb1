"""Three helium-4 atoms in the reference's unit system
(FeynSimul/physical_systems/lm2m2_3part.py:19-153): ``Lm2m2_3part()``.

Units: hbar = m_He = 1, so the 6 coordinates are the Jacobi vectors of three unit masses,
in units of 0.8988882 Angstrom (``xUnit`` in metres, rounded as the reference states it),
and energies are in units of ``potentialUnit`` J (a kernel beta of 1000 is 15 mK).  The
potential is the LM2M2 pair sum; ``energyOp`` is the virial estimator; the radius
operators are about the centre of mass, in coordinate units.  The two numbers that fix the
units (Angstrom per coordinate unit, eV per energy unit) are the reference's, so the same
coordinates give the same values.  ``referenceDerivative=True`` reproduces the reference's
add-on derivative term in ``energyOp`` (see feynsimul_gb300.physical_systems.lm2m2).
"""
from .lm2m2 import _set_unit_cluster

ANGSTROM_PER_UNIT = 0.8988882118208078
EV_PER_UNIT = 773.633685978724


class Lm2m2_3part:
    def __init__(self, referenceDerivative=False):
        self.DOF = 6
        self.groundStateEnergy = -0.126  # K
        self.xUnit = 8.98888e-11         # m
        self.potentialUnit = 2.07098e-22  # J
        _set_unit_cluster(self, 3, ANGSTROM_PER_UNIT, EV_PER_UNIT, referenceDerivative)
