"""Coupled spherical harmonics Y{l1, l2, L, M} of two-electron problems: the index range, the
Clebsch-Gordan coefficients and the selection rules that give a TensorPotential's angular
(row, col) pairs in "Simp" storage.

  CoupledIndex, DefaultCoupledIndexIterator   pyprop/CoupledSphericalHarmonics.py:14-70
  CoupledRange (index list <-> grid index)    core/representation/coupledspherical/coupledrange.h:87-160
  ClebschGordan                               coupledrange.h:17-31 (there through GSL's 3j; here the
                                              Racah formula for the Wigner 3j symbol)
  selection rules, GetBasisPairs              core/tensorpotential/coupledsphericalselectionrule.h:8-183
  geometry names                              pyprop/tensorpotential/basis/CoupledSphericalHarmonic.py:117-139

GetBasisPairs lists every (left, right) grid-index pair whose coupled indices satisfy the rule,
left-major, as the reference's double loop does; the pairs feed gbprop_add_potential's Simp
storage like the reduced-spherical dipole pairs."""
from __future__ import annotations

import math
from collections import namedtuple

import numpy as np

CoupledIndex = namedtuple("CoupledIndex", ["l1", "l2", "L", "M"])


class DefaultCoupledIndexIterator:
    """Every CoupledIndex(l1, l2, L, M) with l1, l2 <= lmax and |l1 - l2| <= L <= l1 + l2 (or all
    combinations when fullTensor), looping M, then L, then l1, then l2
    (pyprop/CoupledSphericalHarmonics.py:40-65).  L defaults to 0..lmax, M to 0; single values
    are accepted for both."""

    def __init__(self, lmax, L=None, M=(0,), fullTensor=False):
        if L is None:
            L = range(lmax + 1)
        self.L = list(L) if hasattr(L, "__iter__") else [L]
        self.M = list(M) if hasattr(M, "__iter__") else [M]
        self.lmax = int(lmax)
        self.FullTensor = bool(fullTensor)

    def __iter__(self):
        for curM in self.M:
            for curL in self.L:
                for l1 in range(self.lmax + 1):
                    for l2 in range(self.lmax + 1):
                        if abs(l1 - l2) <= curL <= l1 + l2 or self.FullTensor:
                            yield CoupledIndex(l1, l2, curL, curM)


class CoupledRange:
    """Grid index <-> coupled index (coupledrange.h:87-160)."""

    def __init__(self, indices):
        self.IndexList = [CoupledIndex(*c) for c in indices]
        self.IndexMap = {c: i for i, c in enumerate(self.IndexList)}
        if len(self.IndexMap) != len(self.IndexList):
            raise ValueError("a coupled index appears twice in the range")

    def Count(self):
        return len(self.IndexList)

    def GetCoupledIndex(self, i):
        return self.IndexList[i]

    def GetGridIndex(self, c):
        return self.IndexMap[CoupledIndex(*c)]


def wigner_3j(j1, j2, j3, m1, m2, m3):
    """The Wigner 3j symbol (j1 j2 j3; m1 m2 m3) for integer arguments, by the Racah formula."""
    if m1 + m2 + m3 != 0 or not (abs(j1 - j2) <= j3 <= j1 + j2):
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    f = math.factorial
    tri = f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3) / f(j1 + j2 + j3 + 1)
    pre = math.sqrt(tri * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3))
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = 0.0
    for k in range(kmin, kmax + 1):
        s += (-1) ** k / (f(k) * f(j1 + j2 - j3 - k) * f(j1 - m1 - k) * f(j2 + m2 - k)
                          * f(j3 - j2 + m1 + k) * f(j3 - j1 - m2 + k))
    return (-1) ** (j1 - j2 - m3) * pre * s


def clebsch_gordan(l1, l2, m1, m2, L, M):
    """<l1 m1 l2 m2 | L M> = (-1)^(M + l1 - l2) sqrt(2L + 1) (l1 l2 L; m1 m2 -M) (coupledrange.h:17-31)."""
    return (-1.0) ** (M + l1 - l2) * math.sqrt(2 * L + 1.0) * wigner_3j(l1, l2, L, m1, m2, -M)


class SelectionRuleDiagonal:
    """coupledsphericalselectionrule.h:172-181: the same (l1, l2, L, M)."""

    def __call__(self, left, right):
        return left == right


class SelectionRuleLinearPolarizedField:
    """coupledsphericalselectionrule.h:149-170: a dipole in a linearly polarized field changes L
    by one at fixed M, and one electron's l by one while the other's stays."""

    def __call__(self, left, right):
        if abs(left.L - right.L) == 1 and left.M == right.M:
            if abs(left.l1 - right.l1) == 1 and left.l2 == right.l2:
                return True
            if abs(left.l2 - right.l2) == 1 and left.l1 == right.l1:
                return True
        return False


class SelectionRuleR12Old:
    """coupledsphericalselectionrule.h:58-83: the same L and M, both triangle conditions."""

    def __call__(self, a, b):
        return (a.L == b.L and a.M == b.M and a.L <= a.l1 + a.l2 and abs(a.l1 - a.l2) <= a.L
                and a.L <= b.l1 + b.l2 and abs(b.l1 - b.l2) <= b.L)


class SelectionRuleR12:
    """coupledsphericalselectionrule.h:86-146: as R12Old, and the electron-electron multipole sum
    over l3 (up to the multipole cutoff) of the four Clebsch-Gordan products is non-zero."""

    def __init__(self, multipoleCutoff=None):
        self.MultipoleCutoff = multipoleCutoff

    def __call__(self, left, right):
        if not SelectionRuleR12Old()(left, right):
            return False
        Lp, Mp, l1p, l2p = left.L, left.M, left.l1, left.l2
        L, M, l1, l2 = right.L, right.M, right.l1, right.l2
        min_l3 = max(abs(l1 - l1p), abs(l2 - l2p))
        max_l3 = min(l1 + l1p, l2 + l2p)
        if self.MultipoleCutoff is not None:
            max_l3 = min(self.MultipoleCutoff, max_l3)
        stop = max(l1, l1p, l2, l2p)
        total = 0.0
        for l3 in range(min_l3, max_l3 + 1):
            for m1p in range(-stop, stop + 1):
                m2p = M - m1p
                for m1 in range(-stop, stop + 1):
                    m2 = M - m1
                    m3 = m1 - m1p
                    cur = (clebsch_gordan(l1p, l2p, m1p, m2p, L, M) * clebsch_gordan(l1, l2, m1, m2, L, M)
                           * clebsch_gordan(l1p, l1, -m1p, m1, l3, m3) * clebsch_gordan(l2p, l2, -m2p, m2, l3, -m3)
                           * (-1.0) ** (m1p + m2p + m3))
                    total += cur
        return abs(total) > 1e-14


def basis_pairs(coupled_range, rule):
    """(npairs, 2) int32 (left, right) grid-index pairs satisfying the rule, left-major
    (CoupledSphericalSelectionRule::GetBasisPairs, coupledsphericalselectionrule.h:16-50)."""
    n = coupled_range.Count()
    out = [(i, j) for i in range(n) for j in range(n)
           if rule(coupled_range.GetCoupledIndex(i), coupled_range.GetCoupledIndex(j))]
    return np.array(out, dtype=np.int32).reshape(-1, 2)


def selection_rule(geometry_name):
    """The rule a coupled-spherical geometry name selects (CoupledSphericalHarmonic.py:117-139)."""
    geom = geometry_name.lower().strip()
    if geom == "diagonal":
        return SelectionRuleDiagonal()
    if geom.startswith("selectionrule_"):
        name = geom[len("selectionrule_"):]
        if name == "r12":
            return SelectionRuleR12Old()
        if name.startswith("r12"):
            return SelectionRuleR12(int(name[4:]))
        if name == "linearpolarizedfield":
            return SelectionRuleLinearPolarizedField()
    raise ValueError("geometry %r not supported by the coupled spherical harmonic basis" % geometry_name)


class GeometryInfoCoupledSphericalHarmonic:
    """Angular storage "Simp" with the pairs of a selection rule
    (GeometryInfoCoupledSphericalHarmonic, CoupledSphericalHarmonic.py:5-31)."""

    def __init__(self, coupled_range, rule):
        self.Range = coupled_range
        self.SelectionRule = rule
        self.IndexPairs = None

    def GetBasisPairs(self):
        if self.IndexPairs is None:
            self.IndexPairs = basis_pairs(self.Range, self.SelectionRule)
        return self.IndexPairs

    def GetGlobalBasisPairCount(self):
        return self.GetBasisPairs().shape[0]

    def GetStorageId(self):
        return "Simp"
