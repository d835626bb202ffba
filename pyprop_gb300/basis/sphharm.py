"""Reduced spherical harmonic angular basis (fixed m), setup only.

Restates ReducedSphericalTools (core/transform/reducedspherical/reducedsphericaltools.cpp:270-360):
  theta grid  = arccos of the (lmax+1)-point Gauss-Legendre nodes, weights = GL weights
  basis       = sqrt(2 pi) * N_lm * P_l^m(cos theta), normalised so that
                sum_q P_l(q) P_l'(q) w_q = delta_ll'
  "derivative" table (differentiation0 = 1), reducedsphericaltools.cpp:349-354:
                l cos(theta) P_l - (l+m) sqrt((2l+1)/(2l-1) (l-|m|)/(l+|m|)) P_{l-1}
Pair tables and projection:
  GeometryInfoReducedSphHarmSelectionRule.GetBasisPairs
      pyprop/tensorpotential/basis/ReducedSphericalHarmonic.py:22-37
  RepresentPotentialInBasisReducedSphericalHarmonic
      core/tensorpotential/basis_reducedspherical.h:11-73
"""
from __future__ import annotations

import math
import numpy as np

from .bspline import gauss_legendre


def assoc_legendre(lmax, m, x):
    """P_l^m(x) for l = |m|..lmax (Condon-Shortley phase included), shape (len(x), lmax+1-|m|)."""
    m = abs(m)
    x = np.asarray(x, dtype=float)
    out = np.zeros((len(x), lmax + 1 - m))
    pmm = np.ones_like(x)
    if m > 0:
        somx2 = np.sqrt((1.0 - x) * (1.0 + x))
        fact = 1.0
        for _ in range(m):
            pmm = -pmm * fact * somx2
            fact += 2.0
    out[:, 0] = pmm
    if lmax > m:
        pmmp1 = x * (2 * m + 1) * pmm
        out[:, 1] = pmmp1
        for l in range(m + 2, lmax + 1):
            pll = (x * (2 * l - 1) * pmmp1 - (l + m - 1) * pmm) / (l - m)
            out[:, l - m] = pll
            pmm, pmmp1 = pmmp1, pll
    return out


class ReducedSphericalTools:
    """Angular quadrature and normalised Legendre tables for fixed m."""

    def __init__(self, lmax, m=0):
        self.lmax = int(lmax)
        self.m = int(m)
        x, w = gauss_legendre(self.lmax + 1)
        self.theta = np.arccos(x)
        self.weights = w
        am = abs(self.m)
        leg = assoc_legendre(self.lmax, self.m, np.cos(self.theta))
        nlc = self.lmax + 1 - am
        self.legendre = np.zeros((len(x), nlc))
        self.legendre_derivative = np.zeros((len(x), nlc))
        for l in range(am, self.lmax + 1):
            li = l - am
            sign = (-1.0) ** self.m if self.m > 0 else 1.0
            norm = sign * math.sqrt(((2.0 * l + 1) / (4 * math.pi)) * (math.factorial(l - am) / math.factorial(l + am)))
            norm *= math.sqrt(2 * math.pi)
            self.legendre[:, li] = leg[:, li] * norm
            if li > 0:
                normalization = math.sqrt((2 * l + 1.0) / (2 * l - 1.0) * (l - am) / float(l + am))
                self.legendre_derivative[:, li] = (l * np.cos(self.theta) * self.legendre[:, li]
                                                   - (l + self.m) * normalization * self.legendre[:, li - 1])

    @property
    def size(self):
        """ReducedSphericalTools::GetSize (reducedsphericaltools.h:53)."""
        return self.lmax - abs(self.m)

    def lvalues(self):
        return np.arange(abs(self.m), self.lmax + 1)


def selection_rule_pairs(tools):
    """Dipole selection-rule pairs (l, l-1), (l, l+1) in the reference order."""
    count = tools.size + 1
    pairs = []
    for i in range(count):
        if i > 0:
            pairs.append((i, i - 1))
        if i < count - 1:
            pairs.append((i, i + 1))
    return np.array(pairs, dtype=np.int32).reshape(-1, 2)


def project_angular(tools, values_theta, pairs, differentiation):
    """sum_q P_row(q) * V(q, ...) * P^(d)_col(q) * w_q for every pair.
    values_theta has the theta index first; returns shape (npairs, ...)."""
    left = tools.legendre
    if differentiation == 0:
        right = tools.legendre
    elif differentiation == 1:
        right = tools.legendre_derivative
    else:
        raise RuntimeError("Reduced spherical harmonics does not support higher derivatives than 1")
    v = np.asarray(values_theta)
    out = np.zeros((len(pairs),) + v.shape[1:], dtype=np.result_type(v.dtype, np.float64))
    for p, (row, col) in enumerate(pairs):
        acc = 0
        for q in range(len(tools.weights)):
            acc = acc + left[q, row] * v[q] * right[q, col] * tools.weights[q]
        out[p] = acc
    return out
