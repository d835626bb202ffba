"""ExpokitPropagator (adaptive Krylov sub-steps with local error control): the CPU
restatement against dense expm, and the GPU propagator (the INI surface of the
reference's KrylovPropagator) against the restatement."""
import numpy as np
import pytest
import scipy.linalg as sl

from helpers import config_text, rel
from oracle import oracle as orc


def _problem(device, m=10, tol=1e-10, norm=None, **kw):
    import pyprop_gb300 as pp
    text = config_text(m=m, **kw).replace("propagator = PamPropagator", "propagator = ExpokitPropagator")
    text = text.replace("krylov_basis_size = %d" % m,
                        "krylov_basis_size = %d\nkrylov_tolerance = %r\nkrylov_norm = %r" % (m, tol, norm or 1e3))
    prob = pp.Problem(pp.LoadString(text), device=device)
    if device == "cpu":
        prob.SetupWavefunction()
    else:
        prob.SetupStep()
    return prob


def _dense(op, s):
    U = op.dense_U()
    Ui = np.linalg.inv(U)
    return U, Ui, Ui.conj().T @ op.dense_potential(s) @ Ui


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_oracle_expokit_meets_its_tolerance(tol):
    prob = _problem("cpu", maxl=3, xsize=30)
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().copy()
    s, dt = 0.3, 0.05
    U, Ui, A = _dense(op, s)
    want = (Ui @ sl.expm(-1j * dt * A) @ (U @ psi0.ravel())).reshape(psi0.shape)
    got, st = op.expokit_advance(psi0, 10, dt, [s], tol, np.linalg.norm(A, np.inf))
    assert rel(got, want) < 100 * tol
    assert st.substeps >= 1 and st.matvecs >= 11


def test_oracle_expokit_imaginary_time_and_breakdown():
    prob = _problem("cpu", maxl=1, xsize=12, order=5)
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().copy()
    U, Ui, A = _dense(op, 0.0)
    x = U @ psi0.ravel()
    want = (Ui @ sl.expm(-0.05 * A) @ x).reshape(psi0.shape)
    got, _ = op.expokit_advance(psi0, 8, -0.05j, [0.0], 1e-10, np.linalg.norm(A, np.inf))
    assert rel(got, want) < 1e-8
    # Krylov dimension >= the problem size: happy breakdown, exact in one sub-step
    n = op.nl * op.nr
    got, st = op.expokit_advance(psi0, n, 0.05, [0.0], 1e-10, np.linalg.norm(A, np.inf))
    want = (Ui @ sl.expm(-1j * 0.05 * A) @ x).reshape(psi0.shape)
    assert rel(got, want) < 1e-11 and st.substeps == 1


@pytest.mark.gpu
@pytest.mark.parametrize("tol", [1e-7, 1e-11])
def test_gpu_expokit_vs_oracle(tol):
    prob = _problem("cuda", m=12, tol=tol, norm=2e3, maxl=4, xsize=40)
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().copy()
    times = [0.0, 0.01, 0.02]
    bp = prob.Propagator.BasePropagator
    scal = [bp._scaling(t) for t in times]
    want, sto = op.expokit_advance(psi0, 12, prob.TimeStep, scal, tol, 2e3)
    prob.Propagator.AdvanceSteps(times, prob.TimeStep)
    got = prob.psi.GetDataNumpy()
    st = prob.Propagator.Statistics
    # the basis is orthogonalised twice (classical Gram-Schmidt) instead of by modified
    # Gram-Schmidt: the same sub-step decisions, results equal to rounding
    assert st.substeps == sto.substeps and st.rejections == sto.rejections
    assert rel(got, want) < 1e-10
    # and the result meets the tolerance against the exact exponential
    U, Ui, _ = _dense(op, 0.0)
    x = U @ psi0.ravel()
    for s in scal:
        A = Ui.conj().T @ op.dense_potential(s) @ Ui
        x = sl.expm(-1j * prob.TimeStep * A) @ x
    assert rel(got, (Ui @ x).reshape(psi0.shape)) < 1000 * tol


@pytest.mark.gpu
def test_gpu_expokit_stable_where_pamp_is_not():
    """A stiff basis with a step far beyond pAMP's reach: Expokit sub-steps keep the
    propagation unitary (norm conserved) and accurate."""
    prob = _problem("cuda", m=12, tol=1e-9, norm=5e4, maxl=6, xsize=60, dt=0.05)
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().copy()
    prob.Propagator.AdvanceSteps([0.0, 0.05], 0.05)
    got = prob.psi.GetDataNumpy()
    U, Ui, _ = _dense(op, 0.0)
    x = U @ psi0.ravel()
    bp = prob.Propagator.BasePropagator
    for t in (0.0, 0.05):
        A = Ui.conj().T @ op.dense_potential(bp._scaling(t)) @ Ui
        x = sl.expm(-1j * 0.05 * A) @ x
    assert rel(got, (Ui @ x).reshape(psi0.shape)) < 1e-6
    assert prob.Propagator.Statistics.substeps > 2
