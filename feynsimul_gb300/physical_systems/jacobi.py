"""Jacobi coordinates of point masses (the reference's FeynSimul/physical_systems/jacobi.py:3-36).

``jacobiCoord(x, m)``: the mass-scaled Jacobi vectors of positions x[0..n-1] (numbers, numpy
arrays or sympy expressions) with masses m:
  jx[0]   = (x[0] - x[1]) sqrt(m0 m1 / (m0 + m1)),
  jx[i]   = (centre of mass of x[0..i] - x[i+1]) sqrt(M_i m_{i+1} / M_{i+1}),  0 < i < n-1,
  jx[n-1] = (centre of mass of all) sqrt(M),
with M_i the mass of particles 0..i.  The map is orthogonal up to the mass scaling, so the
kinetic energy is |d jx / dt|^2 / 2 and, for equal masses, the first n-1 vectors carry all
relative motion.

``toJacobiCoord(expr, x, m, jx)``: sympy expressions in the per-particle coordinates
x[i][d] rewritten in the Jacobi symbols jx[i][d] (needs sympy).
"""


def _sqrt(v):
    try:
        import sympy
        if isinstance(v, sympy.Basic):
            return sympy.sqrt(v)
    except ImportError:
        pass
    import numpy as np
    return np.sqrt(v)


def jacobiCoord(x, m):
    n = len(m)
    if n < 2:
        raise ValueError("at least two particles")
    cum = [m[0]]
    for i in range(1, n):
        cum.append(cum[-1] + m[i])

    def centre(k):  # centre of mass of particles 0..k
        s = x[0] * m[0]
        for j in range(1, k + 1):
            s = s + x[j] * m[j]
        return s / cum[k]

    jx = []
    for i in range(n):
        if i == 0:
            jx.append((x[0] - x[1]) * _sqrt(m[0] * m[1] / (m[0] + m[1])))
        elif i == n - 1:
            jx.append(centre(n - 1) * _sqrt(cum[n - 1]))
        else:
            jx.append((centre(i) - x[i + 1]) * _sqrt(cum[i] * m[i + 1] / cum[i + 1]))
    return jx


def toJacobiCoord(expr, x, m, jx):
    """[sympy expressions in x[i][d]] -> the same expressions in the Jacobi symbols jx[i][d]."""
    import sympy
    n = len(m)
    # coefficient matrix of the linear map, one spatial dimension at a time
    e = [sympy.Integer(1) if i == j else sympy.Integer(0) for i in range(n) for j in range(n)]
    cols = [jacobiCoord([e[i * n + j] for i in range(n)], m) for j in range(n)]
    C = sympy.Matrix(n, n, lambda i, j: cols[j][i])
    Cinv = sympy.simplify(C.inv())
    rep = {}
    for d in range(len(x[0])):
        for i in range(n):
            rep[x[i][d]] = sum(Cinv[i, k] * jx[k][d] for k in range(n))
    return [sympy.sympify(ex).subs(rep, simultaneous=True) for ex in expr]
