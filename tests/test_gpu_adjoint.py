"""Adjoint gradient of bound-state populations with respect to 64 piecewise-linear
field samples, on the GPU, against the dense discrete adjoint and against central
finite differences (h = 1e-6) of the GPU forward propagation."""
import numpy as np
import pytest

from helpers import rel
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

NSTEPS, NSAMPLES = 120, 64


def _setup(checkpoint=50):
    from pyprop_gb300.adjoint import AdjointPropagator, bound_states
    from pyprop_gb300.batch import HydrogenProblem
    prob = HydrogenProblem(lmax=2, nr=24, rmax=20.0, m=16, dt=0.05, seed=7)
    states, _, _ = bound_states(prob)
    psi0 = states[0].reshape(prob.nl, prob.nr)
    rng = np.random.default_rng(11)
    c = 0.6 * np.sin(np.linspace(0, 3 * np.pi, NSAMPLES)) + 0.2 * rng.standard_normal(NSAMPLES)
    ap = AdjointPropagator(prob, NSTEPS, NSAMPLES, checkpoint=checkpoint)
    return prob, states, psi0, c, ap


def _oracle(prob):
    pots = [dict(kind=orc.ORC_DIAG_BANDNH, data=prob.static, pairs=None, timedep=False),
            dict(kind=orc.ORC_SIMP_BANDNH, data=prob.dipole, pairs=prob.pairs, timedep=True)]
    return orc.Operator(prob.nl, prob.nr, prob.kd, prob.kb, prob.cholesky_band().astype(np.complex128), pots)


def test_adjoint_gradient_matches_dense_discrete_adjoint():
    prob, states, psi0, c, ap = _setup()
    psi_T = ap.forward(psi0, c)
    g, dOds = ap.gradient(psi_T, states)
    O = ap.observable(psi_T, states)
    s = ap.scalings(c)
    O_ref, g_ref_s, psi_ref = orc.dense_adjoint_gradient(_oracle(prob), psi0, prob.dt, s, states)
    assert rel(psi_T.cpu().numpy(), psi_ref) < 1e-10
    assert abs(O - O_ref) < 1e-10
    assert 0.05 < O < 0.999                      # the field moves population out of the bound states
    assert rel(dOds, g_ref_s) < 1e-8, rel(dOds, g_ref_s)
    assert rel(g, ap.W.T @ g_ref_s) < 1e-8


def test_adjoint_gradient_matches_central_differences():
    prob, states, psi0, c, ap = _setup()
    psi_T = ap.forward(psi0, c)
    g, _ = ap.gradient(psi_T, states)
    h = 1e-6
    scale = np.abs(g).max()
    for k in (0, 9, 31, 50, 63):
        cp, cm = c.copy(), c.copy()
        cp[k] += h
        cm[k] -= h
        Op = ap.observable(ap.forward(psi0, cp, keep=False), states)
        Om = ap.observable(ap.forward(psi0, cm, keep=False), states)
        fd = (Op - Om) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * scale, (k, fd, g[k])


def test_checkpoint_interval_does_not_change_the_gradient():
    _, states, psi0, c, ap50 = _setup(checkpoint=50)
    g50, _ = ap50.gradient(ap50.forward(psi0, c), states)
    _, _, _, _, ap7 = _setup(checkpoint=7)
    g7, _ = ap7.gradient(ap7.forward(psi0, c), states)
    _, _, _, _, apall = _setup(checkpoint=NSTEPS)
    gall, _ = apall.gradient(apall.forward(psi0, c), states)
    assert rel(g7, g50) < 1e-13
    assert rel(gall, g50) < 1e-13


def test_autograd_function_backward():
    import torch
    from pyprop_gb300.adjoint import ObservableFunction
    _, states, psi0, c, ap = _setup()
    x = torch.tensor(c, dtype=torch.float64, requires_grad=True)
    O = ObservableFunction.apply(x, ap, psi0, states)
    (3.0 * O).backward()
    g, _ = ap.gradient(ap.forward(psi0, c), states)
    assert rel(x.grad.numpy(), 3.0 * g) < 1e-13


def test_autograd_two_forward_calls_then_backward_on_the_first():
    """Two losses through one propagator: backward() of the first call uses that call's own
    checkpoints and field values, not those of the later forward call."""
    import torch
    from pyprop_gb300.adjoint import ObservableFunction
    _, states, psi0, c, ap = _setup()
    c2 = 1.3 * c[::-1].copy()
    x1 = torch.tensor(c, dtype=torch.float64, requires_grad=True)
    x2 = torch.tensor(c2, dtype=torch.float64, requires_grad=True)
    O1 = ObservableFunction.apply(x1, ap, psi0, states)
    O2 = ObservableFunction.apply(x2, ap, psi0, states)
    O1.backward()
    O2.backward()
    g1, _ = ap.gradient(ap.forward(psi0, c), states)
    g2, _ = ap.gradient(ap.forward(psi0, c2), states)
    assert rel(g1, g2) > 1e-3                       # the two calls have different gradients
    assert rel(x1.grad.numpy(), g1) < 1e-13
    assert rel(x2.grad.numpy(), g2) < 1e-13


def test_adjoint_at_reduced_size_vs_central_differences_and_taylor_remainder():
    """l = 0..15 x 200 B-splines (r_max = 100), m = 20, 1000 steps of dt = 0.002, 64 field
    samples: the gradient of the ground-state survival probability against central differences
    and through the Taylor remainder O(c + h d) - O(c) - h g.d, which must fall as h^2.

    The smallest useful difference step is set by the forward map's rounding: the 1000 steps
    leave O with noise of ~1e-13 between nearby field values (not smooth below that), which is
    ~4e-5 of max|g| * 2h at h = 1e-6 and ~1e-7 at h = 1e-4."""
    from pyprop_gb300.adjoint import AdjointPropagator, bound_states
    from pyprop_gb300.batch import HydrogenProblem
    prob = HydrogenProblem(lmax=15, nr=200, rmax=100.0, m=20, dt=0.002, seed=20261205)
    states, _, _ = bound_states(prob)
    ground = states[:1]
    psi0 = states[0].reshape(prob.nl, prob.nr)
    rng = np.random.default_rng(20261205)
    c = rng.normal(0.05, 0.01, NSAMPLES)
    ap = AdjointPropagator(prob, 1000, NSAMPLES, checkpoint=50)
    g, _ = ap.gradient(ap.forward(psi0, c), ground)
    scale = float(np.abs(g).max())

    def O(x):
        return ap.observable(ap.forward(psi0, x, keep=False), ground)

    h = 1e-4
    for k in (5, 31, 58):
        cp, cm = c.copy(), c.copy()
        cp[k] += h
        cm[k] -= h
        fd = (O(cp) - O(cm)) / (2 * h)
        print("sample %d: central difference %.12e, adjoint %.12e" % (k, fd, g[k]))
        assert abs(fd - g[k]) <= 1e-5 * scale, (k, fd, g[k])
    d = rng.standard_normal(NSAMPLES)
    O0, gd = O(c), float(g @ d)
    r1, r2 = [], []
    for hh in (1e-2, 5e-3, 2.5e-3):
        Oh = O(c + hh * d)
        r1.append(abs(Oh - O0))
        r2.append(abs(Oh - O0 - hh * gd))
    print("Taylor remainders: without gradient", r1, "with gradient", r2)
    for a, b in zip(r2, r2[1:]):
        assert 3.0 < a / b < 5.0                    # second order: halving h divides by 4
    for a, b in zip(r1, r1[1:]):
        assert 1.6 < a / b < 2.4                    # first order without the gradient term
