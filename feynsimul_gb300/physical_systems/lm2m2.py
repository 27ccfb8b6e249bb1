"""Helium-4 clusters with the LM2M2 pair potential, as plugin objects.

Counterpart of the reference's FeynSimul/physical_systems/lm2m2_cluster.py:6-95 (which
builds the same system with sympy, Python 2) and lm2m2.h:17-147 (the pair potential).
This module writes the C code itself:

* pair potential: Aziz & Slaman (1991) LM2M2, in Kelvin for r in Angstrom,
  V(r) = eps [A exp(-alpha x + beta x^2) - F(x) (c6/x^6 + c8/x^8 + c10/x^10) + Va(x)],
  x = r / r_m, F(x) = exp(-(D/x - 1)^2) for x < D (else 1), add-on
  Va(x) = A_a (sin(2 pi (x - x1)/(x2 - x1) - pi/2) + 1) on x1 <= x <= x2;
* coordinates: mass-scaled Jacobi vectors of n equal masses (lm2m2_cluster.py:69 and
  jacobi.py:3-36): xi_0 = (r_0 - r_1) sqrt(m/2),
  xi_k = (mean(r_0..r_k) - r_{k+1}) sqrt((k+1) m / (k+2)); the centre of mass drops
  out, leaving DOF = 3 (n - 1), so the kinetic term is |d xi / d tau|^2 / 2;
* units (lm2m2_cluster.py:21-28): length Angstrom, energy Kelvin, beta = 1 / T, and
  m = M_He * (1 Angstrom)^2 k_B / hbar^2;
* operators: the virial energy V + (1/2) sum_k x_k dV/dx_k (lm2m2_cluster.py:75-76), which
  for pair potentials of r^2 is sum_pairs [V + r^2 dV/d(r^2)]; the sum of squared pair
  distances (:79-82); and the pair distances themselves for the pair-distance histogram.

The reference's derivative routine adds 1.0 inside the add-on term
(lm2m2.h:143, ``Aa*(cos(...)*B+1.0)``), which is not the derivative of Va; its energy
estimator is therefore biased for pairs with x1 <= x <= x2.  ``referenceDerivative=True``
reproduces that form for comparisons; the default uses the correct derivative.
"""
from __future__ import annotations

import numpy as np

HE_MASS = 6.64647617e-27  # kg (lm2m2_cluster.py:21)
HBAR = 1.05457148e-34      # J s
KB = 1.3806503e-23         # J / K

# LM2M2 parameters (Aziz & Slaman 1991)
EPS_K = 10.97
RM = 2.9695
A_STAR = 1.89635353e5
ALPHA = 10.70203539
BETA_STAR = -1.90740649
C6, C8, C10 = 1.34687065, 0.41308398, 0.17060159
D_CUT = 1.4088
A_ADD = 0.0026
X1_ADD, X2_ADD = 1.003535949, 1.454790369

# Ground-state energies quoted by the reference for n = 3..10 (lm2m2_cluster.py:17-19),
# magnitudes in K.
GROUND_STATES = [0.0872, 0.387, 0.901, 1.605, 2.478, 3.489, 4.641, 5.904]


def lm2m2_c_code(reference_derivative: bool = False, branchless: bool = True) -> str:
    """C source of lm2m2_r2(r^2) [K] and dlm2m2_dr2(r^2) = dV/d(r^2) [K / Angstrom^2].

    ``branchless`` (default) evaluates every term and selects, so the lanes of a warp
    never diverge on a pair's distance regime: one rsqrt gives r and 1/x^2, the damping
    exp(-(D/x - 1)^2) is taken with D/x - 1 clamped at 0 (F = 1 beyond D), and the add-on
    Aa (sin(B(x - x1) - pi/2) + 1) = Aa (1 - cos(B(x - x1))) is masked outside [x1, x2].
    ``branchless=False`` gives the reference-shaped form with branches (lm2m2.h:22-147)."""
    if branchless:
        return _lm2m2_c_code_branchless(reference_derivative)
    add_term = "(cs * B + 1.0)" if reference_derivative else "(cs * B)"
    return f"""
inline FLOAT_TYPE fs_sq(FLOAT_TYPE v) {{ return v * v; }}
inline FLOAT_TYPE lm2m2_r2(FLOAT_TYPE r2)
{{
    FLOAT_TYPE x = sqrt(r2) * {1.0 / RM!r};
    FLOAT_TYPE ix2 = 1.0 / (x * x);
    FLOAT_TYPE rat = ((({C10!r} * ix2 + {C8!r}) * ix2) + {C6!r}) * ix2 * ix2 * ix2;
    if (x < {D_CUT!r}) {{
        if (x > {0.0005 / RM!r}) {{
            FLOAT_TYPE q = {D_CUT!r} / x - 1.0;
            rat = rat * exp(-q * q);
        }} else {{
            rat = 0.0;
        }}
    }}
    FLOAT_TYPE v = {A_STAR!r} * exp(x * ({BETA_STAR!r} * x - {ALPHA!r})) - rat;
    if (x >= {X1_ADD!r} && x <= {X2_ADD!r}) {{
        FLOAT_TYPE B = {2.0 * np.pi / (X2_ADD - X1_ADD)!r};
        v = v + {A_ADD!r} * (sin(B * (x - {X1_ADD!r}) - M_PI_2) + 1.0);
    }}
    return {EPS_K!r} * v;
}}
inline FLOAT_TYPE dlm2m2_dr2(FLOAT_TYPE r2)
{{
    FLOAT_TYPE r = sqrt(r2);
    FLOAT_TYPE x = r * {1.0 / RM!r};
    FLOAT_TYPE ix = 1.0 / x;
    FLOAT_TYPE ix2 = ix * ix;
    FLOAT_TYPE ix6 = ix2 * ix2 * ix2;
    FLOAT_TYPE rat = (({C10!r} * ix2 + {C8!r}) * ix2 + {C6!r}) * ix6;
    FLOAT_TYPE drat = -((({10.0 * C10!r} * ix2 + {8.0 * C8!r}) * ix2 + {6.0 * C6!r}) * ix6 * ix);
    FLOAT_TYPE dfr;
    if (x < {D_CUT!r}) {{
        if (x > {0.0005 / RM!r}) {{
            FLOAT_TYPE q = {D_CUT!r} * ix - 1.0;
            FLOAT_TYPE F = exp(-q * q);
            dfr = F * drat + F * (2.0 * q * {D_CUT!r} * ix2) * rat;
        }} else {{
            dfr = 0.0;
        }}
    }} else {{
        dfr = drat;
    }}
    FLOAT_TYPE dv = {A_STAR!r} * exp(x * ({BETA_STAR!r} * x - {ALPHA!r})) * ({2.0 * BETA_STAR!r} * x - {ALPHA!r}) - dfr;
    if (x >= {X1_ADD!r} && x <= {X2_ADD!r}) {{
        FLOAT_TYPE B = {2.0 * np.pi / (X2_ADD - X1_ADD)!r};
        FLOAT_TYPE cs = cos(B * (x - {X1_ADD!r}) - M_PI_2);
        dv = dv + {A_ADD!r} * {add_term};
    }}
    return {EPS_K!r} * dv / ({2.0 * RM!r} * r);
}}
"""


def _lm2m2_c_code_branchless(reference_derivative: bool) -> str:
    # Constants are folded where that saves operations: eps and the powers of r_m into every
    # coefficient of V, so it is written in r rather than x = r / r_m, and log2(e) into the
    # exponents (exp(z) = exp2(z log2 e), the form the hardware evaluates):
    # exp(x (beta x - alpha)) = exp2(r (beta' r - alpha')), and the damping
    # exp(-(D/x - 1)^2) = exp2(-q^2) with q = max(D r_m / r - 1, 0) sqrt(log2 e).
    # The FP32 rounding of the folded constants is systematic: it moves a 10-atom cluster's
    # FP32 energy by about 2e-7 relative against FP64.  The derivative, evaluated only by
    # the energy operator, keeps the unfolded form (folded in the same way, it added 1e-6).
    L = float(1.0 / np.log(2.0))
    sL = float(np.sqrt(L))
    rm2 = RM * RM
    dr = D_CUT * RM
    tiny = 0.0005
    B = float(2.0 * np.pi / (X2_ADD - X1_ADD))
    # reference form of the add-on derivative term: Aa (cos(...) B + 1) = Aa (B sin(w) + 1)
    add_d = f"({A_ADD!r} * ({B!r} * sw + 1.0))" if reference_derivative else f"({A_ADD * B!r} * sw)"
    return f"""
inline FLOAT_TYPE fs_sq(FLOAT_TYPE v) {{ return v * v; }}
inline FLOAT_TYPE lm2m2_r2(FLOAT_TYPE r2)
{{
    FLOAT_TYPE ir = rsqrt(r2);
    FLOAT_TYPE r = r2 * ir;
    FLOAT_TYPE u = ir * ir;
    FLOAT_TYPE rat = ((({EPS_K * C10 * RM ** 10!r} * u + {EPS_K * C8 * RM ** 8!r}) * u) + {EPS_K * C6 * RM ** 6!r}) * u * u * u;
    FLOAT_TYPE q = fmax({dr * sL!r} * ir - {sL!r}, 0.0);
    rat = (r2 > {tiny * tiny!r}) ? rat * exp2(-q * q) : 0.0;
    FLOAT_TYPE w = {B / RM!r} * r - {B * X1_ADD!r};
    FLOAT_TYPE add = (r >= {X1_ADD * RM!r} && r <= {X2_ADD * RM!r}) ? {EPS_K * A_ADD!r} : 0.0;
    return {EPS_K * A_STAR!r} * exp2(r * ({L * BETA_STAR / RM ** 2!r} * r - {L * ALPHA / RM!r})) - rat + add * (1.0 - cos(w));
}}
inline FLOAT_TYPE dlm2m2_dr2(FLOAT_TYPE r2)
{{
    FLOAT_TYPE ir = rsqrt(r2);
    FLOAT_TYPE x = r2 * ir * {1.0 / RM!r};
    FLOAT_TYPE ix = {RM!r} * ir;
    FLOAT_TYPE ix2 = ix * ix;
    FLOAT_TYPE ix6 = ix2 * ix2 * ix2;
    FLOAT_TYPE rat = (({C10!r} * ix2 + {C8!r}) * ix2 + {C6!r}) * ix6;
    FLOAT_TYPE drat = -((({10.0 * C10!r} * ix2 + {8.0 * C8!r}) * ix2 + {6.0 * C6!r}) * ix6 * ix);
    FLOAT_TYPE q = fmax({D_CUT!r} * ix - 1.0, 0.0);
    FLOAT_TYPE F = exp(-q * q);
    FLOAT_TYPE dfr = (r2 > {tiny * tiny!r}) ? F * drat + F * (2.0 * q * {D_CUT!r} * ix2) * rat : 0.0;
    FLOAT_TYPE sw = sin({B!r} * (x - {X1_ADD!r}));
    FLOAT_TYPE inwin = (x >= {X1_ADD!r} && x <= {X2_ADD!r}) ? 1.0 : 0.0;
    FLOAT_TYPE dv = {A_STAR!r} * exp(x * ({BETA_STAR!r} * x - {ALPHA!r})) * ({2.0 * BETA_STAR!r} * x - {ALPHA!r})
                    - dfr + inwin * {add_d};
    return {EPS_K!r} * dv * ir * {0.5 / RM!r};
}}
"""


def lm2m2_numpy(r, reference_derivative=False):
    """FP64 numpy evaluation of V(r) [K] and dV/d(r^2), for tests and analysis."""
    r = np.asarray(r, dtype=np.float64)
    x = r / RM
    rat = C6 / x ** 6 + C8 / x ** 8 + C10 / x ** 10
    drat = -6 * C6 / x ** 7 - 8 * C8 / x ** 9 - 10 * C10 / x ** 11
    q = D_CUT / x - 1.0
    F = np.where(x < D_CUT, np.exp(-q * q), 1.0)
    dF = np.where(x < D_CUT, F * 2.0 * q * D_CUT / x ** 2, 0.0)
    tiny = x <= 0.0005 / RM
    frat = np.where(tiny & (x < D_CUT), 0.0, F * rat)
    dfrat = np.where(tiny & (x < D_CUT), 0.0, F * drat + dF * rat)
    base = A_STAR * np.exp(-ALPHA * x + BETA_STAR * x * x)
    vb = base - frat
    dvb = base * (-ALPHA + 2 * BETA_STAR * x) - dfrat
    B = 2 * np.pi / (X2_ADD - X1_ADD)
    win = (x >= X1_ADD) & (x <= X2_ADD)
    va = np.where(win, A_ADD * (np.sin(B * (x - X1_ADD) - np.pi / 2) + 1.0), 0.0)
    cs = np.cos(B * (x - X1_ADD) - np.pi / 2)
    dva = np.where(win, A_ADD * (cs * B + (1.0 if reference_derivative else 0.0)), 0.0)
    v = EPS_K * (vb + va)
    dv_dr2 = EPS_K * (dvb + dva) / (RM * 2.0 * r)
    return v, dv_dr2


def jacobi_matrix(n: int, m: float) -> np.ndarray:
    """J with xi = J r for n equal masses; rows 0..n-2 relative, row n-1 the scaled centre."""
    J = np.zeros((n, n))
    J[0, 0], J[0, 1] = np.sqrt(m / 2.0), -np.sqrt(m / 2.0)
    for k in range(1, n - 1):
        s = np.sqrt((k + 1) * m / (k + 2))
        J[k, :k + 1] = s / (k + 1)
        J[k, k + 1] = -s
    J[n - 1, :] = np.sqrt(n * m) / n
    return J


def _set_cluster_code(obj, n: int, J: np.ndarray, reference_derivative: bool,
                      length_A: float = 1.0, v_scale: float = 1.0) -> None:
    """Plugin code of n LM2M2 atoms in Jacobi coordinates xi = J r.

    Sets obj.J, obj.B (positions relative to the centre of mass from the relative xi),
    obj.pairs, obj.userCode, obj.potential, obj.energyOp (virial energy),
    obj.meanSquaredRadiusOp (sum of squared pair distances [Angstrom^2]) and
    obj.pairDistanceOps (pair distances [Angstrom]).  Coordinates are in units of length_A
    Angstrom; the potential and the energy are v_scale times their value in Kelvin."""
    dof = 3 * (n - 1)
    obj.J = J
    obj.B = np.linalg.inv(J)[:, : n - 1]
    obj.pairs = [(a, b) for a in range(n) for b in range(a + 1, n)]
    BA = obj.B * length_A                 # positions in Angstrom
    xs = [f"x{i + 1}" for i in range(dof)]
    args = ", ".join(f"FLOAT_TYPE {v}" for v in xs)

    def comp(coefs, dim):
        terms = [f"{float(c)!r} * {xs[3 * k + dim]}" for k, c in enumerate(coefs) if abs(c) > 1e-15]
        return " + ".join(terms) if terms else "0.0"

    # pair vectors: straight from the Jacobi coordinates where that takes fewer terms (2-4
    # atoms: the first pair is one Jacobi vector), else positions relative to the centre of
    # mass and their differences
    nnz = lambda v: int(np.sum(np.abs(v) > 1e-15))
    direct = sum(nnz(BA[a] - BA[b]) for (a, b) in obj.pairs)
    via_positions = sum(nnz(BA[a]) for a in range(n)) + len(obj.pairs)
    pos = []
    r2 = {}
    if direct < via_positions:
        for (a, b) in obj.pairs:
            for dim in range(3):
                pos.append(f"    FLOAT_TYPE d{a}_{b}_{dim} = {comp(BA[a] - BA[b], dim)};")
            r2[(a, b)] = " + ".join(f"fs_sq(d{a}_{b}_{dim})" for dim in range(3))
    else:
        for a in range(n):
            for dim in range(3):
                pos.append(f"    FLOAT_TYPE p{a}_{dim} = {comp(BA[a], dim)};")
        for (a, b) in obj.pairs:
            r2[(a, b)] = " + ".join(f"fs_sq(p{a}_{dim} - p{b}_{dim})" for dim in range(3))
    body_pos = "\n".join(pos)
    pot_sum = " + ".join(f"lm2m2_r2({r2[p]})" for p in obj.pairs)
    vir_terms = []
    for i, p in enumerate(obj.pairs):
        vir_terms.append(f"    {{ FLOAT_TYPE q = {r2[p]}; e += lm2m2_r2(q) + q * dlm2m2_dr2(q); }}")
    msr = " + ".join(r2[p] for p in obj.pairs)
    scaled = (lambda e: e) if v_scale == 1.0 else (lambda e: f"{v_scale!r} * ({e})")
    obj.userCode = lm2m2_c_code(reference_derivative) + f"""
inline FLOAT_TYPE lm2m2_cluster_potential({args})
{{
{body_pos}
    return {scaled(pot_sum)};
}}
inline FLOAT_TYPE lm2m2_cluster_virial_energy({args})
{{
{body_pos}
    FLOAT_TYPE e = 0.0;
{chr(10).join(vir_terms)}
    return {scaled("e")};
}}
inline FLOAT_TYPE lm2m2_cluster_pair_r2_sum({args})
{{
{body_pos}
    return {msr};
}}
"""
    call = ", ".join(xs)
    obj.potential = f"lm2m2_cluster_potential({call})"
    obj.energyOp = f"lm2m2_cluster_virial_energy({call})"
    obj.meanSquaredRadiusOp = f"lm2m2_cluster_pair_r2_sum({call})"
    obj.pairDistanceOps = tuple(
        "sqrt(" + " + ".join(
            f"fs_sq({comp(BA[a] - BA[b], dim)})" for dim in range(3)) + ")"
        for (a, b) in obj.pairs)


# Kelvin in electronvolts as the reference's pair-potential routines use it
# (lm2m2_3part.py userCode, lm2m2_4part.py userCode: k = 8.6173324e-5 eV/K)
KB_EV = 8.6173324e-5


def reference_helper_code(eV_per_unit=None) -> str:
    """C helpers under the names the reference's plugins define, for operator strings written
    against them: sqr; lm2m2sqrt(r^2) [K] and dlm2m2sqrtdr(r^2) = d/d(r^2) (lm2m2.h:17-147);
    with ``eV_per_unit`` also lm2m2(r) and dlm2m2dr(r) = d/dr in eV for r in Angstrom (the
    three- and four-atom plugins' userCode).  Requires lm2m2_c_code's functions."""
    code = """
inline FLOAT_TYPE sqr(FLOAT_TYPE v) { return v * v; }
inline FLOAT_TYPE lm2m2sqrt(FLOAT_TYPE sr) { return lm2m2_r2(sr); }
inline FLOAT_TYPE dlm2m2sqrtdr(FLOAT_TYPE sr) { return dlm2m2_dr2(sr); }
"""
    if eV_per_unit is not None:
        code += f"""inline FLOAT_TYPE lm2m2(FLOAT_TYPE r) {{ return {KB_EV!r} * lm2m2_r2(r * r); }}
inline FLOAT_TYPE dlm2m2dr(FLOAT_TYPE r) {{ return {2.0 * KB_EV!r} * r * dlm2m2_dr2(r * r); }}
"""
    return code


def _set_unit_cluster(obj, n: int, angstrom_per_unit: float, eV_per_unit: float,
                      reference_derivative: bool) -> None:
    """n atoms in the units of the reference's three- and four-atom plugins: hbar = m_He = 1,
    so the coordinates are Jacobi vectors of unit masses, in units of angstrom_per_unit
    Angstrom, and the potential is in units of 1 / eV_per_unit eV.  Sets the plugin code and
    the reference's operators (lm2m2_3part.py:26-28, lm2m2_4part.py:31-33): mean squared
    radius and mean radius about the centre of mass, and mean squared pair distance, all in
    coordinate units."""
    _set_cluster_code(obj, n, jacobi_matrix(n, 1.0), reference_derivative,
                      length_A=angstrom_per_unit, v_scale=KB_EV * eV_per_unit)
    obj.pairR2SumOp = obj.meanSquaredRadiusOp            # sum of squared pair distances [A^2]
    obj.userCode += reference_helper_code(eV_per_unit)
    xs = [f"x{i + 1}" for i in range(obj.DOF)]
    sumsq = " + ".join(f"sqr({v})" for v in xs)
    # unit masses: sum_a |p_a - centre|^2 = |xi|^2, and sum over pairs |p_a - p_b|^2 = n |xi|^2
    obj.meanSquaredRadiusOp = f"{1.0 / n!r} * ({sumsq})"
    obj.meanSquaredAtomDistOp = f"{2.0 / (n - 1)!r} * ({sumsq})"

    def comp(coefs, dim):
        terms = [f"{float(c)!r} * {xs[3 * k + dim]}" for k, c in enumerate(coefs) if abs(c) > 1e-15]
        return " + ".join(terms) if terms else "0.0"

    radii = [f"sqrt({' + '.join(f'sqr({comp(obj.B[a], dim)})' for dim in range(3))})" for a in range(n)]
    obj.meanRadiusOp = f"{1.0 / n!r} * ({' + '.join(radii)})"


class Lm2m2Cluster:
    """n helium-4 atoms at temperature T [K] with the LM2M2 pair potential."""

    def __init__(self, n: int, T: float, referenceDerivative: bool = False):
        if n < 2:
            raise Exception("n must be >=2")
        d = 3
        self.n = n
        self.T = float(T)
        self.DOF = (n - 1) * d
        self.rUnit = 1e-10
        self.potentialUnit = KB
        self.beta = self.potentialUnit / (KB * self.T)
        self.m = HE_MASS * self.rUnit ** 2 / HBAR ** 2 * self.potentialUnit
        if 3 <= n <= 10:
            self.groundStateEnergy = -GROUND_STATES[n - 3]
        _set_cluster_code(self, n, jacobi_matrix(n, self.m), referenceDerivative)

    # ---- coordinates -------------------------------------------------------------
    def positions_to_jacobi(self, r):
        """r [..., n, 3] (Angstrom) -> relative Jacobi coordinates [..., DOF]."""
        r = np.asarray(r, dtype=np.float64)
        xi = np.einsum("ij,...jd->...id", self.J, r)[..., : self.n - 1, :]
        return xi.reshape(*r.shape[:-2], self.DOF)

    def jacobi_to_positions(self, x):
        """[..., DOF] -> positions relative to the centre of mass [..., n, 3]."""
        x = np.asarray(x, dtype=np.float64)
        xi = x.reshape(*x.shape[:-1], self.n - 1, 3)
        return np.einsum("ik,...kd->...id", self.B, xi)

    def potential_numpy(self, x):
        pos = self.jacobi_to_positions(x)
        v = 0.0
        for (a, b) in self.pairs:
            rr = np.linalg.norm(pos[..., a, :] - pos[..., b, :], axis=-1)
            v = v + lm2m2_numpy(rr)[0]
        return v

    def initial_paths(self, walkers: int, N: int, rng, side=(3.0, 5.0), noise=0.1):
        """Paths [walkers, DOF*N] (DOF-major): for n = 3 a random equilateral triangle of
        side U(side) with random orientation, otherwise n quasi-uniform points on a sphere
        (Fibonacci lattice) whose closest pair is U(side) apart, randomly oriented; plus
        N(0, noise) Angstrom per slice and coordinate."""
        n = self.n
        L = rng.uniform(side[0], side[1], size=walkers)
        if n == 3:
            base = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, np.sqrt(3) / 2, 0.0]])
        else:
            k = np.arange(n) + 0.5
            z = 1.0 - 2.0 * k / n
            phi = np.pi * (1.0 + np.sqrt(5.0)) * k
            rxy = np.sqrt(1.0 - z * z)
            base = np.stack([rxy * np.cos(phi), rxy * np.sin(phi), z], axis=1)
            dmin = min(np.linalg.norm(base[a] - base[b]) for a in range(n) for b in range(a + 1, n))
            base = base / dmin
        base = base - base.mean(axis=0)
        q = rng.standard_normal((walkers, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        w, x, y, z = q.T
        R = np.stack([
            np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
            np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
            np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)
        r0 = np.einsum("wij,nj->wni", R, base) * L[:, None, None]  # [walkers, n, 3]
        xi0 = self.positions_to_jacobi(r0)                        # [walkers, DOF]
        paths = np.repeat(xi0[:, :, None], N, axis=2)              # [walkers, DOF, N]
        if noise > 0:
            # isotropic Cartesian noise of width `noise` is isotropic noise of width
            # noise*sqrt(m) in mass-scaled Jacobi coordinates (the transformation is
            # sqrt(m) times an orthogonal one for equal masses)
            paths = paths + rng.normal(0.0, noise * np.sqrt(self.m), size=paths.shape)
        return np.ascontiguousarray(paths.reshape(walkers, self.DOF * N))
