"""Four helium-4 atoms in the reference's unit system
(FeynSimul/physical_systems/lm2m2_4part.py:19-158): ``Lm2m2_4part()``.

Units: hbar = m_He = 1, so the 9 coordinates are the Jacobi vectors of four unit masses, in
units of 0.4923414 Angstrom, and energies are in units of ``potentialUnit`` J.  Same
operators and conventions as feynsimul_gb300.physical_systems.lm2m2_3part.
"""
from .lm2m2 import _set_unit_cluster

ANGSTROM_PER_UNIT = 0.49234135028973836
EV_PER_UNIT = 232.09010579361725


class Lm2m2_4part:
    def __init__(self, referenceDerivative=False):
        self.DOF = 9
        self.groundStateEnergy = -0.4              # K
        self.meanSquaredRadius = 7.15 ** 2.0       # Angstrom^2
        self.meanSquaredAtomDist = 10.7 ** 2.0     # Angstrom^2
        self.xUnit = 4.92341e-11                   # m
        self.potentialUnit = 6.90325e-22           # J
        _set_unit_cluster(self, 4, ANGSTROM_PER_UNIT, EV_PER_UNIT, referenceDerivative)
