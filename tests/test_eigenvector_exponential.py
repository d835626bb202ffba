"""krylov_exponentiation_method = 1: pAMP::EigenvectorExponential
(core/krylov/pamp/pamp/pamp.h:567-607, selected in pampwrapper.cpp:56-61).

The oracle restates it with zgeev (numpy.linalg.eig) on A = -i dt H_m and the reference's
W diag(e^lambda) W^H; the GPU forms the same y from a Jacobi eigen-decomposition of the
Hermitian part of H_m.  Both are checked against the Pade path (method 0) and against each
other."""
import numpy as np
import pytest

from helpers import make_problem, rel, scalings_for
from oracle import oracle as orc


def test_oracle_eigenvector_method_matches_pade():
    prob = make_problem(device="cpu", setup=False, maxl=3, xsize=30, m=12, dt=0.01)
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    scal = scalings_for(prob, 10)
    a, _ = op.advance(psi0, 12, prob.TimeStep, scal)
    b, _ = op.advance_eigenvector(psi0, 12, prob.TimeStep, scal)
    assert rel(b, a) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32-mixed", 1e-4)])
@pytest.mark.parametrize("dt", [0.01, -0.02j])
def test_gpu_eigenvector_method_vs_oracle(precision, tol, dt):
    import pyprop_gb300 as pp
    from helpers import config_text
    text = config_text(maxl=3, xsize=30, m=12, dt=dt, precision=precision)
    text = text.replace("krylov_basis_size = 12", "krylov_basis_size = 12\nkrylov_exponentiation_method = 1")
    prob = pp.Problem(pp.LoadString(text))
    prob.SetupStep()
    assert prob.Propagator.ExponentiationMethod == 1
    op = orc.Operator.from_problem(prob)
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    nsteps = 10
    scal = scalings_for(prob, nsteps)
    want, _ = op.advance_eigenvector(psi0, 12, prob.TimeStep, scal)
    prob.AdvanceSteps(nsteps)
    got = prob.psi.GetDataNumpy().astype(np.complex128)
    assert rel(got, want) < tol
    h = prob.Propagator.Handle()
    assert h.stats().last_scaling_order == 0
