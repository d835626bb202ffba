"""Coupled spherical harmonics: index range, Clebsch-Gordan coefficients and selection rules
(pyprop/CoupledSphericalHarmonics.py:14-70, core/tensorpotential/coupledsphericalselectionrule.h).

The 3j symbols are checked against sympy's exact values; the linearly-polarized-field rule
against the dipole matrix elements <l1' l2' L' M| cos(theta_1) + cos(theta_2) |l1 l2 L M> built
from Clebsch-Gordan algebra (every non-zero element lies on a listed pair, and every listed pair
with allowed parities has one); the R12 rule's multipole sum against the same sum with sympy."""
import math

import numpy as np
import pytest

from pyprop_gb300.basis import coupled as cs


def _range(lmax=3, L=(0, 1, 2), M=0):
    return cs.CoupledRange(cs.DefaultCoupledIndexIterator(lmax, L=L, M=M))


def test_default_iterator_order_and_triangle():
    r = _range(2, L=[0, 1])
    idx = r.IndexList
    assert idx[0] == (0, 0, 0, 0) and idx[1] == (1, 1, 0, 0) and idx[2] == (2, 2, 0, 0)   # L = 0 first
    assert all(abs(c.l1 - c.l2) <= c.L <= c.l1 + c.l2 for c in idx)
    # L = 0: l1 = l2 (3); L = 1: (0,1) (1,0) (1,1) (1,2) (2,1) (2,2)
    assert len(idx) == 3 + 6
    full = cs.CoupledRange(cs.DefaultCoupledIndexIterator(2, L=[0, 1], fullTensor=True))
    assert full.Count() == 2 * 9
    assert r.GetGridIndex(r.GetCoupledIndex(5)) == 5


def test_wigner_3j_against_sympy():
    wigner = pytest.importorskip("sympy.physics.wigner")
    rng = np.random.default_rng(3)
    for _ in range(200):
        j1, j2 = int(rng.integers(0, 5)), int(rng.integers(0, 5))
        j3 = int(rng.integers(abs(j1 - j2), j1 + j2 + 1))
        m1, m2 = int(rng.integers(-j1, j1 + 1)), int(rng.integers(-j2, j2 + 1))
        m3 = -m1 - m2
        want = float(wigner.wigner_3j(j1, j2, j3, m1, m2, m3))
        assert abs(cs.wigner_3j(j1, j2, j3, m1, m2, m3) - want) < 1e-13
    # orthonormality of the Clebsch-Gordan coefficients
    l1, l2 = 2, 3
    for L in range(1, 6):
        for Lp in range(1, 6):
            s = sum(cs.clebsch_gordan(l1, l2, m1, 1 - m1, L, 1) * cs.clebsch_gordan(l1, l2, m1, 1 - m1, Lp, 1)
                    for m1 in range(-l1, l1 + 1) if abs(1 - m1) <= l2)
            assert abs(s - (L == Lp)) < 1e-13


def _dipole_element(a, b):
    """<a| cos(theta_1) + cos(theta_2) |b> in the coupled basis, from <l' 0|cos|l 0>-type single
    electron elements <l' m|cos|l m> and Clebsch-Gordan recoupling."""
    def cos_el(lp, l, m):
        if abs(m) > l or abs(m) > lp:
            return 0.0
        if lp == l + 1:
            return math.sqrt(((l + 1) ** 2 - m * m) / ((2 * l + 1) * (2 * l + 3)))
        if lp == l - 1:
            return math.sqrt((l * l - m * m) / ((2 * l - 1) * (2 * l + 1)))
        return 0.0
    if a.M != b.M:
        return 0.0
    tot = 0.0
    for m1 in range(-max(a.l1, b.l1), max(a.l1, b.l1) + 1):
        m2 = a.M - m1
        ca = cs.clebsch_gordan(a.l1, a.l2, m1, m2, a.L, a.M)
        cb = cs.clebsch_gordan(b.l1, b.l2, m1, m2, b.L, b.M)
        if ca == 0.0 or cb == 0.0:
            continue
        e = 0.0
        if a.l2 == b.l2:
            e += cos_el(a.l1, b.l1, m1)
        if a.l1 == b.l1:
            e += cos_el(a.l2, b.l2, m2)
        tot += ca * cb * e
    return tot


def test_linear_polarized_field_pairs_cover_the_dipole():
    r = _range(3, L=(0, 1, 2, 3))
    rule = cs.selection_rule("selectionrule_linearpolarizedfield")
    pairs = {tuple(p) for p in cs.basis_pairs(r, rule)}
    n = r.Count()
    for i in range(n):
        for j in range(n):
            v = _dipole_element(r.GetCoupledIndex(i), r.GetCoupledIndex(j))
            if abs(v) > 1e-12:
                assert (i, j) in pairs, (r.GetCoupledIndex(i), r.GetCoupledIndex(j), v)
    # left-major order, as the reference's double loop
    lst = cs.basis_pairs(r, rule)
    assert np.all(np.diff(lst[:, 0] * n + lst[:, 1]) > 0)
    assert cs.GeometryInfoCoupledSphericalHarmonic(r, rule).GetStorageId() == "Simp"


def test_r12_rules():
    r = _range(2, L=(0, 1))
    old = {tuple(p) for p in cs.basis_pairs(r, cs.selection_rule("selectionrule_r12"))}
    new = {tuple(p) for p in cs.basis_pairs(r, cs.selection_rule("selectionrule_r12_4"))}
    assert new <= old                                      # the multipole sum only removes pairs
    diag = cs.basis_pairs(r, cs.selection_rule("diagonal"))
    assert np.array_equal(diag, np.stack([np.arange(r.Count())] * 2, 1))
    assert all((i, i) in new for i in range(r.Count()))    # 1/r12 has diagonal elements
