"""Renormalization and the overlap-metric observables on the device.

Problem.AdvanceStep normalises psi after every step when the Propagation key
renormalization is true (pyprop/Problem.py:167-168 -> Wavefunction::Normalize,
core/wavefunction.cpp:194-218); here the Krylov propagators do it inside the device step.
Checked against the oracle stepping one step at a time and normalising in the overlap metric
between steps, in imaginary time (where the norm decays and renormalization matters).
Wavefunction.InnerProduct / GetNorm (CombinedRepresentation::InnerProduct,
combinedrepresentation.cpp:423-474) and Problem.GetEnergyExpectationValue (Problem.py:254-276,
with BasisPropagator.MultiplyHamiltonian = S^-1 H, BasisPropagator.py:116-124) run through
libgbprop and are compared with dense numpy restatements."""
import numpy as np
import pytest

from helpers import make_problem, rel, scalings_for

pytestmark = pytest.mark.gpu


def _s_norm2(op, x):
    U = op.dense_U()
    y = U @ x.ravel()
    return float(np.vdot(y, y).real)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32-mixed", 1e-5)])
def test_imaginary_time_with_renormalization_vs_oracle(precision, tol):
    from oracle import oracle as orc
    prob = make_problem(maxl=3, xsize=30, m=10, dt=-0.02j, renorm=True, precision=precision)
    op = orc.Operator.from_problem(prob)
    psi = prob.psi.GetDataNumpy().astype(np.complex128)
    nsteps = 25
    scal = scalings_for(prob, nsteps)
    for k in range(nsteps):
        psi, _ = op.advance(psi, prob.Propagator.BasisSize, prob.TimeStep, scal[k:k + 1])
        psi = psi / np.sqrt(_s_norm2(op, psi))
    for _ in range(5):                                   # AdvanceStep, one step at a time
        prob.AdvanceStep()
    prob.AdvanceSteps(nsteps - 5)                        # one device call for the rest
    got = prob.psi.GetDataNumpy().astype(np.complex128)
    assert rel(got, psi) < tol
    assert abs(prob.psi.GetNorm() - 1.0) < (1e-13 if precision == "fp64" else 1e-6)


def test_inner_product_and_energy_vs_dense():
    from oracle import oracle as orc
    prob = make_problem(maxl=3, xsize=30, m=10)
    op = orc.Operator.from_problem(prob)
    rng = np.random.default_rng(17)
    a = rng.standard_normal((op.nl, op.nr)) + 1j * rng.standard_normal((op.nl, op.nr))
    b = rng.standard_normal((op.nl, op.nr)) + 1j * rng.standard_normal((op.nl, op.nr))
    U = op.dense_U()
    S = U.conj().T @ U
    wa, wb = prob.psi.Copy(), prob.psi.Copy()
    wa.SetData(a)
    wb.SetData(b)
    want = np.vdot(a.ravel(), S @ b.ravel())
    got = wa.InnerProduct(wb)
    assert abs(got - want) < 1e-13 * abs(want)
    assert abs(wa.GetNorm() - np.sqrt(np.vdot(a.ravel(), S @ a.ravel()).real)) < 1e-13 * wa.GetNorm()
    # <psi|H(t)|psi> / <psi|S|psi> at the problem's time
    prob.PropagatedTime = 37.0
    s = prob.Propagator.BasePropagator._scaling(37.0)
    H = op.dense_potential(s)
    psi = prob.psi.GetDataNumpy().ravel()
    e_want = (np.vdot(psi, H @ psi) / np.vdot(psi, S @ psi)).real
    assert abs(prob.GetEnergyExpectationValue() - e_want) < 1e-11 * abs(e_want)


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_device_populations_vs_host(precision):
    """Bound-state populations and ionisation evaluated on the GPU against the host restatement."""
    import torch
    from pyprop_gb300 import observables as ob
    prob = make_problem(maxl=3, xsize=30, m=10, precision=precision)
    states, _, _ = ob.problem_bound_states(prob)
    S = ob.radial_overlap(prob)
    prob.AdvanceSteps(5)
    psi = prob.psi.GetData()
    dev = ob.DevicePopulations(states, S, prob.Propagator.Handle())
    got = dev.report(psi)
    want = ob.report(prob.psi.GetDataNumpy().astype(np.complex128), states, S)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.abs(got["populations"] - want["populations"]).max() < tol
    assert abs(got["ionisation"] - want["ionisation"]) < tol and abs(got["norm"] - want["norm"]) < tol
