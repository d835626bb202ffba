"""Radial TensorPotential set-up on the GPU (gbprop_bspline_bands) against the host restatement
(pyprop_gb300/basis/bspline.py band_diagonals / band_cholesky_upper_diagonals, itself pinned to
the reference's quadrature, knot and breakpoint modules by tests/golden/setup_golden.npz): the
same recursions, quadrature and summation order, so the matrices agree to the last bit or to a
few ulps."""
import numpy as np
import pytest

from pyprop_gb300.basis import bspline as bs

pytestmark = pytest.mark.gpu

TERMS = [(0, 0, 1.0), (0, 2, -0.5), (2, 0, 1.0), (1, 0, -1.0), (0, 1, 1.0), (1, 0, 1.0)]


def _host(basis):
    g = basis.grid
    fs = [np.ones(len(g)), np.full(len(g), -0.5), 1.0 / (2.0 * g * g), -1.0 / g, np.ones(len(g)), 1.0 / g]
    ders = [0, 2, 0, 0, 1, 0]
    return [basis.band_diagonals(f, d) for f, d in zip(fs, ders)]


@pytest.mark.parametrize("kind,order,n", [("linear", 7, 106), ("explinear", 7, 1000), ("linear", 3, 40),
                                          ("linear", 9, 300), ("exponential", 5, 80)])
def test_bspline_bands_match_host(kind, order, n):
    from pyprop_gb300 import _native
    if kind == "linear":
        bps = bs.linear_breakpoints(0.0, 50.0, n - order + 4)
    elif kind == "exponential":
        bps = bs.exponential_breakpoints(0.0, 60.0, n - order + 4, 3.0)
    else:
        bps = bs.make_breakpoints("exponentiallinear", 0.0, 400.0, 70, gamma=1.5, xpartition=15.0)
    basis = bs.BSplineBasis(bps, order, bs.continuity_sequence(len(bps), order, "zero"))
    want = _host(basis)
    got, U = _native.bspline_bands(basis, TERMS, cholesky=True)
    for w, g in zip(want, got):
        scale = np.abs(w).max()
        assert np.abs(g - w).max() <= 4e-16 * scale
    Uh = bs.band_cholesky_upper_diagonals(want[0], order - 1)
    assert np.abs(U - Uh).max() <= 4e-16 * np.abs(Uh).max()


def test_hydrogen_problem_gpu_setup_matches_host():
    from pyprop_gb300.batch import HydrogenProblem
    a = HydrogenProblem(lmax=9, nr=300, rmax=100.0, m=12, seed=3, setup="host")
    b = HydrogenProblem(lmax=9, nr=300, rmax=100.0, m=12, seed=3, setup="gpu")
    for x, y in ((a.static, b.static), (a.dipole, b.dipole), (a.Sdiag, b.Sdiag), (a.Ud, b.Ud)):
        assert np.abs(x - y).max() <= 4e-16 * np.abs(x).max()
