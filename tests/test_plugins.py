"""The reference-named plugin modules (physical_systems/lm2m2_3part.py, lm2m2_4part.py,
lm2m2_cluster.py, jacobi.py, partSys.py) against the reference's own expressions.

plugins_ref.npz holds the reference's three- and four-atom plugin expressions evaluated in
FP64 from their C strings (tests/golden/make_golden.py); the plugins here are generated
by this package's own code, evaluated the same way.  The reference writes some Jacobi
coefficients with 8 digits, hence the 1e-6 relative tolerance."""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN
from plugin_c import eval_exprs

ATTRS = ("potential", "energyOp", "meanSquaredRadiusOp", "meanRadiusOp", "meanSquaredAtomDistOp")


@pytest.mark.parametrize("module,cls", [("lm2m2_3part", "Lm2m2_3part"), ("lm2m2_4part", "Lm2m2_4part")])
def test_few_atom_plugins_match_reference_expressions(module, cls):
    import importlib
    z = np.load(os.path.join(GOLDEN, "plugins_ref.npz"))
    x, want = z[f"{module}_x"], z[f"{module}_values"]
    mod = importlib.import_module(f"feynsimul_gb300.physical_systems.{module}")
    sysm = getattr(mod, cls)(referenceDerivative=True)   # the reference's add-on derivative form
    assert sysm.DOF == x.shape[1]
    got = eval_exprs(sysm.userCode, [getattr(sysm, a) for a in ATTRS], sysm.DOF, x)
    for j, a in enumerate(ATTRS):
        scale = np.abs(want[:, j]).max()
        np.testing.assert_allclose(got[:, j], want[:, j], rtol=1e-6, atol=1e-9 * scale, err_msg=a)
    # the default virial operator differs only by the add-on derivative term
    plain = getattr(mod, cls)()
    g2 = eval_exprs(plain.userCode, [plain.potential], plain.DOF, x)
    np.testing.assert_allclose(g2[:, 0], want[:, 0], rtol=1e-6, atol=1e-9 * np.abs(want[:, 0]).max())


def test_reference_helper_names_in_user_code():
    """Operator strings written against the reference's helpers compile and agree."""
    from feynsimul_gb300.physical_systems.lm2m2 import lm2m2_numpy
    from feynsimul_gb300.physical_systems.lm2m2_3part import Lm2m2_3part
    from feynsimul_gb300.physical_systems.lm2m2_cluster import Lm2m2_cluster
    r = np.array([[2.5], [3.0], [4.0], [7.0]])
    c = Lm2m2_cluster(3, 1.0)
    v = eval_exprs(c.userCode, ["lm2m2sqrt(sqr(x1))", "dlm2m2sqrtdr(x1 * x1)"], 1, r)
    v_np, dv_np = lm2m2_numpy(r[:, 0])
    np.testing.assert_allclose(v[:, 0], v_np, rtol=1e-12)
    np.testing.assert_allclose(v[:, 1], dv_np, rtol=1e-12)
    t = Lm2m2_3part()
    ev = eval_exprs(t.userCode, ["lm2m2(x1)"], 1, r)
    np.testing.assert_allclose(ev[:, 0], 8.6173324e-5 * v_np, rtol=1e-12)   # eV


def test_cluster_alias_keeps_reference_signature():
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    from feynsimul_gb300.physical_systems.lm2m2_cluster import Lm2m2_cluster
    a = Lm2m2_cluster(4, 0.5, useJacobi=True, simplify=False, verbose=False, enableDouble=True)
    b = Lm2m2Cluster(4, 0.5)
    assert (a.DOF, a.beta, a.m) == (b.DOF, b.beta, b.m)
    assert a.potential == b.potential and a.energyOp == b.energyOp
    assert a.groundStateEnergy == 0.387        # the reference stores the magnitude
    with pytest.raises(Exception, match="jacobi"):
        Lm2m2_cluster(3, 1.0, useJacobi=False)
    with pytest.raises(Exception):
        Lm2m2_cluster(1, 1.0)


def test_jacobi_coordinates():
    from feynsimul_gb300.physical_systems import jacobi
    from feynsimul_gb300.physical_systems.lm2m2 import jacobi_matrix
    rng = np.random.RandomState(3)
    for n in (2, 3, 5):
        x = [rng.randn(3) for _ in range(n)]
        np.testing.assert_allclose(np.array(jacobi.jacobiCoord(x, [2.5] * n)), jacobi_matrix(n, 2.5) @ np.array(x))
    # unequal masses: orthogonal up to the mass scaling (sum m |x|^2 is preserved)
    m = [1.0, 3.0, 0.5, 2.0]
    x = [rng.randn(3) for _ in m]
    jx = np.array(jacobi.jacobiCoord(x, m))
    assert np.isclose((jx ** 2).sum(), sum(mi * (xi ** 2).sum() for mi, xi in zip(m, x)))
    sympy = pytest.importorskip("sympy")
    xs = [[sympy.Symbol(f"r{i}_{d}") for d in range(3)] for i in range(3)]
    js = [[sympy.Symbol(f"x{i * 3 + d + 1}") for d in range(3)] for i in range(3)]
    mm = [sympy.Symbol("m", positive=True)] * 3
    ex = jacobi.toJacobiCoord([sum((xs[0][d] - xs[2][d]) ** 2 for d in range(3))], xs, mm, js)[0]
    num = {s: v for s, v in zip(sum(xs, []), rng.randn(9))}
    jv = np.array(jacobi.jacobiCoord([np.array([num[s] for s in row]) for row in xs], [1.7] * 3))
    sub = {mm[0]: 1.7, **{js[i][d]: jv[i][d] for i in range(3) for d in range(3)}}
    assert np.isclose(float(ex.subs(sub)), sum((num[xs[0][d]] - num[xs[2][d]]) ** 2 for d in range(3)))


def test_hyper_radial_potential():
    from feynsimul_gb300.physical_systems.partSys import getHyperRadialPotential
    x = [0.0, 1.0, 3.0, 6.0]
    d = lambda a, b: (a - b) ** 2
    two = sum(d(x[i], x[j]) for i in range(4) for j in range(i + 1, 4))
    v = getHyperRadialPotential(x, d, [lambda s: s, lambda s: 0.0 * s, lambda s: 100.0 * s])
    assert np.isclose(v, two + 100.0 * two)


def test_new_plugins_compile_for_the_gpu():
    """Each plugin builds into a sweep kernel (NVRTC, no GPU needed)."""
    import ctypes
    from feynsimul_gb300 import _lib as L
    from feynsimul_gb300.physical_systems.lm2m2_3part import Lm2m2_3part
    from feynsimul_gb300.physical_systems.lm2m2_4part import Lm2m2_4part
    from feynsimul_gb300.physical_systems.lm2m2_cluster import Lm2m2_cluster
    for s in (Lm2m2_3part(), Lm2m2_4part(), Lm2m2_cluster(5, 1.0)):
        cfg = L.FsConfig()
        for k, v in dict(dof=s.DOF, n_slices=64, bisection_level=2, beta=2.0, n_walkers=64, walkers_per_group=1,
                         operator_runs=1, metro_steps_per_operator_run=1, enable_parallelize_path=1,
                         luxury_factor=2, ranlux_int_max=2 ** 32 - 1, accum=1, fast_math=1).items():
            setattr(cfg, k, v)
        ops = [s.energyOp] + [getattr(s, a) for a in ("meanSquaredRadiusOp", "meanRadiusOp",
                                                       "meanSquaredAtomDistOp") if hasattr(s, a)]
        o, no = L.strings(ops)
        c, nc = L.strings([])
        h, nh = L.strings([])
        buf = ctypes.create_string_buffer(1 << 16)
        rc = L.lib().fs_compile_only(ctypes.byref(cfg), s.potential.encode(), s.userCode.encode(), o, no, c, nc,
                                     h, nh, buf, len(buf))
        assert rc == 0, buf.value.decode()[-2000:]
