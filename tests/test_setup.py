"""Setup path (B-spline and angular bases, TensorPotential generation, config
parsing) against the reference's own setup modules (golden fixtures) and
analytic anchors."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

import pyprop_gb300 as pp
from pyprop_gb300.basis import bspline as bs
from pyprop_gb300.basis import sphharm as sph
from pyprop_gb300.tensorpotential import bandnh_pairs, bandnh_to_dense, dense_to_bandnh

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "setup_golden.npz"))


@pytest.mark.parametrize("order", [2, 3, 5, 7, 9, 10, 11, 16])
def test_gauss_legendre_golden(order):
    n, w = bs.gauss_legendre(order)
    assert np.allclose(n, GOLD["gl_nodes_%d" % order], atol=5e-15, rtol=0)
    assert np.allclose(w, GOLD["gl_weights_%d" % order], atol=5e-15, rtol=0)


def test_breakpoints_golden():
    assert np.allclose(bs.linear_breakpoints(0.0, 50.0, 103), GOLD["bp_linear"], rtol=1e-15)
    assert np.allclose(bs.exponential_breakpoints(0.0, 100.0, 60, 3.0), GOLD["bp_exponential"], rtol=1e-14)
    ref = GOLD["bp_explinear"]
    got = bs.exponential_linear_breakpoints(0.0, 20.0, 400.0, 60, 2.0)
    assert got.shape == ref.shape and np.allclose(got, ref, rtol=1e-13)


@pytest.mark.parametrize("case", ["small", "vanilla", "custom", "explinear"])
def test_bspline_object_golden(case):
    g = lambda k: GOLD["bs_%s_%s" % (case, k)]
    cfg = {k[len("bs_%s_cfg_" % case):]: GOLD[k][()] for k in GOLD.files if k.startswith("bs_%s_cfg_" % case)}
    cfg = {k: (v.item() if hasattr(v, "item") else v) for k, v in cfg.items()}
    sec = pp.Section("RadialRepresentation")
    for k, v in cfg.items():
        sec.Set(k, str(v) if isinstance(v, (str, np.str_)) else v)
    b = bs.bspline_from_section(sec)
    assert np.allclose(b.breakpoints, g("bp"), rtol=1e-13)
    assert np.array_equal(b.continuity, g("cont"))
    assert np.allclose(b.knots, g("knots"), rtol=1e-13)
    assert b.count == int(g("count"))
    assert np.allclose(b.grid, g("grid"), rtol=1e-13, atol=1e-13)
    assert np.allclose(b.grid_weights, g("gw"), rtol=1e-12)


def test_workload_basis_sizes():
    # configuration of the CPU-runnable workload: 106 B-splines
    assert int(GOLD["bs_small_count"]) == 106


def test_hydrogen_bound_states():
    b = bs.BSplineBasis(bs.linear_breakpoints(0.0, 50.0, 103), 7, bs.continuity_sequence(103, 7, "zero"))
    S = b.overlap()
    K = b.band_matrix(np.full(len(b.grid), -0.5), 2)
    R1 = b.band_matrix(-1.0 / b.grid, 0)
    R2 = b.band_matrix(1.0 / b.grid ** 2, 0)
    for l, want in ((0, [-0.5, -0.125]), (1, [-0.125, -1 / 18.0])):
        e = sl.eigh(K + R1 + l * (l + 1) / 2.0 * R2, S, eigvals_only=True)
        assert np.allclose(e[:2], want, atol=2e-9)


def test_bspline_partition_of_unity_and_derivatives():
    bps = bs.linear_breakpoints(0.0, 10.0, 12)
    b = bs.BSplineBasis(bps, 5, bs.continuity_sequence(12, 5, "vanilla"))
    B, D1, D2 = b.tables()
    assert np.allclose(B.sum(0), 1.0, atol=1e-14)
    assert np.allclose(D1.sum(0), 0.0, atol=1e-12)
    assert np.allclose(D2.sum(0), 0.0, atol=1e-10)
    # swap rule: first-derivative matrix with constant weight is antisymmetric
    zb = bs.BSplineBasis(bps, 5, bs.continuity_sequence(12, 5, "zero"))
    D = zb.band_matrix(np.ones(len(zb.grid)), 1)
    assert np.allclose(D, -D.T, atol=1e-13)


def test_angular_couplings_closed_form():
    t = sph.ReducedSphericalTools(9, 0)
    assert np.allclose(t.legendre.T @ np.diag(t.weights) @ t.legendre, np.eye(10), atol=1e-13)
    pairs = sph.selection_rule_pairs(t)
    assert len(pairs) == 2 * 9 and tuple(pairs[0]) == (0, 1) and tuple(pairs[1]) == (1, 0)
    vals = sph.project_angular(t, np.cos(t.theta)[:, None], pairs, 0)[:, 0]
    for (r, c), v in zip(pairs, vals):
        l = min(r, c)
        assert abs(v - (l + 1) / np.sqrt((2 * l + 1) * (2 * l + 3))) < 1e-14


def test_bandnh_layout_roundtrip():
    rng = np.random.default_rng(3)
    n, k = 9, 2
    M = np.zeros((n, n), dtype=np.complex128)
    for d in range(-k, k + 1):
        M += np.diag(rng.standard_normal(n - abs(d)) + 1j * rng.standard_normal(n - abs(d)), d)
    v = dense_to_bandnh(M, k)
    assert np.array_equal(bandnh_to_dense(v, n, k), M)
    pairs = bandnh_pairs(n, k)
    W = 2 * k + 1
    for i in range(n):
        for j in range(max(0, i - k), min(n, i + k + 1)):
            assert tuple(pairs[j * W + k + i - j]) == (i, j)


def test_config_parsing_base_interpolation_import(tmp_path):
    (tmp_path / "inc.ini").write_text("[Shared]\nvalue = 3\n")
    (tmp_path / "main.ini").write_text(
        "[Import]\nfiles = ['inc.ini']\n\n[Pulse]\nfrequency = 0.5\ncycles = 4\n"
        "pulse_duration = 2 * pi / %(frequency)s * %(cycles)s\n\n"
        "[Propagation]\nbase = \"Pulse\"\ntimestep = 0.01 + 0.0j\nlist = [1, 2]\n")
    conf = pp.Load(str(tmp_path / "main.ini"))
    assert conf.Shared.value == 3
    assert abs(conf.Propagation.pulse_duration - 2 * np.pi / 0.5 * 4) < 1e-12
    assert conf.Propagation.timestep == 0.01 and conf.Propagation.list == [1, 2]


def test_problem_setup_consolidation(small_problem_cpu):
    pots = small_problem_cpu.Propagator.BasePropagator.PotentialList
    assert [p.GetStorageIds() for p in pots] == [["Diag", "BandNH"], ["Simp", "BandNH"]]
    static, laser = pots
    assert not static.IsTimeDependent and laser.IsTimeDependent
    assert static.PotentialData.shape == (10, 13 * 106)
    assert laser.PotentialData.shape == (18, 13 * 106)
    assert np.all(laser.PotentialData.real == 0)       # velocity gauge terms are purely imaginary
    assert np.all(static.PotentialData.imag == 0)
    assert abs(small_problem_cpu.psi.GetNorm() - 1.0) < 1e-13


def test_laser_function_values():
    conf = pp.Load(os.path.join(os.path.dirname(__file__), "..", "pyprop_gb300", "configs",
                                "hydrogen_velocity_small.ini"))
    sec = conf.LaserPotentialVelocityBase
    T = sec.pulse_duration
    assert pp.LaserFunctionVelocity(sec, -1.0) == 0.0 and pp.LaserFunctionVelocity(sec, T) == 0.0
    t = 0.3 * T
    want = sec.amplitude * np.sin(np.pi * t / T) ** 2 * -np.cos(sec.frequency * t)
    assert abs(pp.LaserFunctionVelocity(sec, t) - want) < 1e-15


GEO = np.load(os.path.join(os.path.dirname(__file__), "golden", "geometry_golden.npz"))


@pytest.mark.parametrize("n,k", [(9, 2), (20, 6), (103, 6), (5, 6), (1, 0)])
def test_bandnh_pairs_golden(n, k):
    """BandNH storage order against the reference's own GeometryInfoCommonBandedNonHermitian
    (GeometryInfo.py:433-454), run by tests/golden/make_golden.py."""
    from pyprop_gb300.tensorpotential import bandnh_pairs
    np.testing.assert_array_equal(bandnh_pairs(n, k), GEO["bandnh_pairs_%d_%d" % (n, k)])


@pytest.mark.parametrize("lmax,m", [(3, 0), (9, 0), (63, 0), (5, 2), (1, 0)])
def test_dipole_selection_pairs_golden(lmax, m):
    """Dipole selection-rule pairs against the reference's own
    GeometryInfoReducedSphHarmSelectionRule (basis/ReducedSphericalHarmonic.py:5-45)."""
    from pyprop_gb300.basis.sphharm import ReducedSphericalTools, selection_rule_pairs
    got = selection_rule_pairs(ReducedSphericalTools(lmax, m))
    np.testing.assert_array_equal(got, GEO["selection_pairs_%d_%d" % (lmax, m)])
    assert len(got) == int(GEO["selection_count_%d_%d" % (lmax, m)])


LASER = np.load(os.path.join(os.path.dirname(__file__), "golden", "laser_golden.npz"))


@pytest.mark.parametrize("case", ["nophase", "phase"])
def test_laser_function_golden(case):
    """The velocity-gauge pulse against the reference's own LaserFunctionVelocity
    (examples/tensor/helium_stabilization_sae/example.py:220-230), including both pulse edges."""
    class Sec:
        pass
    sec = Sec()
    prefix = "laser_%s_cfg_" % case
    for k in LASER.files:
        if k.startswith(prefix):
            setattr(sec, k[len(prefix):], float(LASER[k]))
    got = np.array([pp.LaserFunctionVelocity(sec, t) for t in LASER["laser_%s_t" % case]])
    np.testing.assert_allclose(got, LASER["laser_%s_f" % case], rtol=1e-14, atol=1e-17)
