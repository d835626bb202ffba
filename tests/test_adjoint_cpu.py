"""CPU checks of the gradient machinery: the dense discrete adjoint (the reference
result for the GPU adjoint) against finite differences, the augmented block operator against
scipy's Frechet derivative through the CPU oracle, the field-sample weights and the
bound states used as the observable."""
import numpy as np
import pytest

from helpers import rel
from oracle import oracle as orc


def _problem(**kw):
    from pyprop_gb300.batch import HydrogenProblem
    args = dict(lmax=2, nr=24, rmax=20.0, m=16, dt=0.05, seed=7)
    args.update(kw)
    return HydrogenProblem(**args)


def _oracle(prob):
    pots = [dict(kind=orc.ORC_DIAG_BANDNH, data=prob.static, pairs=None, timedep=False),
            dict(kind=orc.ORC_SIMP_BANDNH, data=prob.dipole, pairs=prob.pairs, timedep=True)]
    return orc.Operator(prob.nl, prob.nr, prob.kd, prob.kb, prob.cholesky_band().astype(np.complex128), pots)


def test_hat_weights_interpolate_linear_functions():
    from pyprop_gb300.adjoint import hat_weights
    T, K = 3.0, 7
    t = np.linspace(0, T, 41)
    W = hat_weights(t, T, K)
    assert np.allclose(W.sum(1), 1.0)
    c = 0.3 + 1.7 * np.linspace(0, T, K)          # samples of a linear function
    assert np.allclose(W @ c, 0.3 + 1.7 * t)
    assert np.count_nonzero(W, axis=1).max() <= 2


def test_bound_states_are_hydrogen_levels():
    from pyprop_gb300.adjoint import bound_states
    prob = _problem(lmax=1, nr=60, rmax=40.0)
    states, e, ls = bound_states(prob)
    e0 = e[ls == 0]
    assert abs(e0[0] + 0.5) < 1e-6
    assert abs(e0[1] + 0.125) < 1e-4
    assert abs(e[ls == 1][0] + 0.125) < 1e-4
    # normalised in the overlap metric and orthogonal
    S = np.kron(np.eye(prob.nl), _dense_S(prob))
    G = states.conj() @ S @ states.T
    assert np.allclose(G, np.eye(len(states)), atol=1e-10)


def _dense_S(prob):
    S = np.zeros((prob.nr, prob.nr))
    for d in range(-prob.kd, prob.kd + 1):
        i = np.arange(max(0, -d), min(prob.nr, prob.nr - d))
        S[i, i + d] = prob.Sdiag[prob.kd + d, i]
    return S


def test_dense_gradient_matches_central_differences():
    from pyprop_gb300.adjoint import bound_states
    prob = _problem()
    op = _oracle(prob)
    states, _, _ = bound_states(prob)
    psi0 = states[0].reshape(prob.nl, prob.nr)
    rng = np.random.default_rng(3)
    s = 0.8 * rng.standard_normal(12)
    O, g, _ = orc.dense_adjoint_gradient(op, psi0, prob.dt, s, states)
    h = 1e-6
    for n in (0, 5, 11):
        sp, sm = s.copy(), s.copy()
        sp[n] += h
        sm[n] -= h
        fd = (orc.dense_adjoint_gradient(op, psi0, prob.dt, sp, states)[0]
              - orc.dense_adjoint_gradient(op, psi0, prob.dt, sm, states)[0]) / (2 * h)
        assert abs(fd - g[n]) <= 1e-6 * max(1.0, abs(g).max()), (n, fd, g[n])


def test_augmented_operator_gives_frechet_derivative():
    """One pAMP step of the 2*nl-row block operator from [0; psi] gives
    [d(step)/ds psi; step psi] (CPU oracle vs scipy expm_frechet)."""
    import scipy.linalg as sl
    from pyprop_gb300 import _native
    from pyprop_gb300.adjoint import AugmentedOperator
    prob = _problem()
    kinds = {_native.STORAGE_DIAG: orc.ORC_DIAG_BANDNH, _native.STORAGE_SIMP: orc.ORC_SIMP_BANDNH}
    pots = [dict(kind=kinds[st], data=d, pairs=p, timedep=td) for st, p, d, td in AugmentedOperator.potentials(prob)]
    aug = orc.Operator(2 * prob.nl, prob.nr, prob.kd, prob.kb, prob.cholesky_band().astype(np.complex128), pots)
    op = _oracle(prob)
    psi = prob.initial_state()
    s = 0.37
    x = np.zeros((2 * prob.nl, prob.nr), dtype=np.complex128)
    x[prob.nl:] = psi
    got, _ = aug.advance(x, 40, prob.dt, [s])
    U = op.dense_U()
    Ui = np.linalg.inv(U)
    H0 = op.dense_potential(0.0)
    H1 = op.dense_potential(1.0) - H0
    A = Ui.conj().T @ (H0 + s * H1) @ Ui
    A1 = Ui.conj().T @ H1 @ Ui
    E, L = sl.expm_frechet(-1j * prob.dt * A, -1j * prob.dt * A1)
    want_d = (Ui @ L @ U @ psi.ravel()).reshape(psi.shape)
    want_e = (Ui @ E @ U @ psi.ravel()).reshape(psi.shape)
    assert rel(got[prob.nl:], want_e) < 1e-11
    assert rel(got[:prob.nl], want_d) < 1e-9
