"""Several time-dependent TensorPotentials with distinct time functions.

The reference scales every consolidated potential by its own time function, evaluated with
its own config section (pyprop/tensorpotential/TensorPotential.py:98-100, looped over by
pyprop/propagator/Propagator.py:61-66); only potentials sharing one function are consolidated
(TensorPotential.py:128-163).  Here one dipole part runs on a second pulse
(LaserFunctionSimpleLength at another frequency), so two time functions remain after
consolidation."""
import numpy as np
import pytest

from helpers import config_text, rel, step_times

pytestmark = []


def _two_pulse_config(precision="fp64"):
    text = config_text(maxl=4, xsize=34, m=10, dt=0.02, precision=precision)
    old = "[LaserPotentialVelocity2]\nbase = \"LaserPotentialVelocityBase\"\n"
    assert old in text
    return text.replace(old, old + "time_function = LaserFunctionSimpleLength\nfrequency = 0.113\n"
                                   "amplitude = 0.4\n")


def _problem(device, precision="fp64"):
    import pyprop_gb300 as pp
    prob = pp.Problem(pp.LoadString(_two_pulse_config(precision)), device=device)
    if device == "cpu":
        prob.SetupWavefunction()
    else:
        prob.SetupStep()
    return prob


def _scalings(prob, n):
    bp = prob.Propagator.BasePropagator
    # mid-pulse, where both functions are non-zero
    return np.array([bp._scalings_at(t + 60.0) for t in step_times(prob, n)])


def test_two_time_functions_after_consolidation():
    from pyprop_gb300.propagator import time_function_numbers
    prob = _problem("cpu")
    pots = prob.Propagator.BasePropagator.PotentialList
    assert time_function_numbers(pots) == [0, 1, 2]
    s = _scalings(prob, 3)
    assert s.shape == (3, 2) and np.all(s != 0.0) and not np.allclose(s[:, 0], s[:, 1])


def test_oracle_scales_each_potential_by_its_function():
    from oracle import oracle as orc
    prob = _problem("cpu")
    op = orc.Operator.from_problem(prob)
    assert op.nfuncs == 2
    rng = np.random.default_rng(5)
    x = rng.standard_normal((op.nl, op.nr)) + 1j * rng.standard_normal((op.nl, op.nr))
    s = np.array([0.3, -1.7])
    dense = op.dense_potential(s)
    assert rel(op.multiply_potentials(x, s), (dense @ x.ravel()).reshape(x.shape)) < 1e-14
    # the sum of the two single-function operators
    d1, d2, d0 = op.dense_potential([1.0, 0.0]), op.dense_potential([0.0, 1.0]), op.dense_potential([0.0, 0.0])
    assert np.allclose(dense, d0 + 0.3 * (d1 - d0) - 1.7 * (d2 - d0), rtol=0, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_two_time_functions_vs_oracle(precision):
    import torch
    from oracle import oracle as orc
    prob = _problem("cuda", precision)
    h = prob.Propagator.Handle()
    assert h.nfuncs == 2
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    nsteps = 20
    scal = _scalings(prob, nsteps)
    want, _ = op.advance(psi0, prob.Propagator.BasisSize, prob.TimeStep, scal)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    d = torch.as_tensor(psi0).to("cuda", cdt)
    h.advance(d, scal, prob.TimeStep)
    h.synchronize()
    err = rel(d.cpu().numpy().astype(np.complex128), want)
    assert err < (1e-11 if precision == "fp64" else 1e-4), err
    # the matvec at the step's two values
    src = torch.as_tensor(psi0).to("cuda", cdt)
    dst = torch.zeros_like(src)
    h.matvec(src, dst, scal[3], balanced=True)
    wmv = op.balanced_matvec(psi0, scal[3])
    assert rel(dst.cpu().numpy().astype(np.complex128), wmv) < (1e-13 if precision == "fp64" else 1e-5)
    # Problem.AdvanceStep evaluates both functions at PropagatedTime
    prob.psi.SetData(psi0)
    prob.PropagatedTime = 60.0
    for _ in range(3):
        prob.AdvanceStep()
    want3, _ = op.advance(psi0, prob.Propagator.BasisSize, prob.TimeStep, scal[:3])
    assert rel(prob.psi.GetDataNumpy().astype(np.complex128), want3) < (1e-11 if precision == "fp64" else 1e-4)
