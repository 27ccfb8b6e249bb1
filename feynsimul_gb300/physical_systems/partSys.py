"""Few-body potentials from hyper-radii (the reference's FeynSimul/physical_systems/partSys.py:2-12).

``getHyperRadialPotential(x, distFun, interactions)``: interactions[k] is a (k+2)-body term, a
function of the hyper-squared-radius of k+2 particles, i.e. the sum of distFun over their
pairs.  The potential is the sum of every k-body term over all k-particle subsets of x.
Works on numbers, numpy arrays or sympy expressions.
"""
from itertools import combinations


def getHyperRadialPotential(x, distFun, interactions):
    def hyper_sqr_radius(ps):
        total = 0
        for a, b in combinations(ps, 2):
            total = total + distFun(a, b)
        return total

    total = 0
    for k, interaction in enumerate(interactions):
        for subset in combinations(range(len(x)), k + 2):
            total = total + interaction(hyper_sqr_radius([x[p] for p in subset]))
    return total
