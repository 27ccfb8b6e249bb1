"""1D harmonic oscillator plugin, V(x) = k x^2 / 2 (FeynSimul/physical_systems/harm_osc.py:34-53)."""


class HarmOsc:
    def __init__(self, k=1.0, lb=False):
        """Potential and virial energy operator of V = k x^2 / 2.

        ``lb`` selects the higher-order (eps-corrected) potential and energy operator of the
        reference's lb variant; ``eps`` is the time step macro every kernel defines."""
        self.potential = "0.5 * " + str(k) + " * x1 * x1"
        if lb:
            self.potential = "0.5 * (1.0 + sqr(eps)/12.0)*sqr(x1)"
        self.userCode = "FLOAT_TYPE sqr(FLOAT_TYPE x){return x*x;}"
        self.energyOp = str(k) + " * x1 * x1"
        if lb:
            self.energyOp = "2.0 * 0.5*(1.0 + sqr(eps)/4.0)*sqr(x1)"
        self.DOF = 1
