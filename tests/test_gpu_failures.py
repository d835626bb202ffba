"""Device-side failures reach the caller through the C ABI and the Python surface.

The reference throws as soon as its Pade LU fails (core/krylov/pamp/pamp/pamp.h:544-550);
here the kernels record a failure in the handle's control block and return, and the host
reports it (gbprop.h, gbprop_advance):
  * NaN in the wavefunction          -> GBPROP_ENONFINITE
  * a bounded device wait gives up   -> GBPROP_ETIMEOUT  (the handle's wait limit set so that
                                        the staging wait and the grid barrier give up at once)
  * a singular Pade denominator      -> GBPROP_ELU       (zgetrf's info != 0, injected by the host)
None of these faults or hangs the GPU.  Each failure is reported once, and afterwards the same
handle propagates the seeded start exactly as the oracle does."""
import numpy as np
import pytest

from helpers import make_problem, rel, scalings_for
from oracle import oracle as orc
from pyprop_gb300 import _native

pytestmark = pytest.mark.gpu

ENONFINITE, ETIMEOUT, ELU = 4, 5, 6
PRECS = ["fp64", "fp32-mixed"]
# FP64: the parity bar; FP32-mixed: the complex64 budget of a few steps from a random start
TOL = {"fp64": 1e-11, "fp32-mixed": 1e-4}


def _problem(precision):
    return make_problem(precision=precision, maxl=3, xsize=30, m=8, dt=0.01)


def _recovers(prob, precision, psi0):
    """Three steps from psi0 on the same handle agree with the oracle."""
    import torch
    nsteps = 3
    scal = scalings_for(prob, nsteps)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    d = torch.as_tensor(psi0).to("cuda", cdt)
    h = prob.Propagator.Handle()
    h.advance(d, scal, prob.TimeStep)
    h.synchronize()
    op = orc.Operator.from_problem(prob)
    want, _ = op.advance(psi0.astype(np.complex128), prob.Propagator.BasisSize, prob.TimeStep, list(scal))
    assert rel(d.cpu().numpy().astype(np.complex128), want) < TOL[precision]


@pytest.mark.parametrize("precision", PRECS)
def test_nonfinite_wavefunction(precision):
    import torch
    prob = _problem(precision)
    psi0 = prob.psi.GetDataNumpy().copy()
    h = prob.Propagator.Handle()
    bad = psi0.copy()
    bad[1, 5] = np.nan
    prob.psi.SetData(bad)
    prob.AdvanceStep()
    with pytest.raises(_native.GbpropError) as e:
        h.synchronize()
    assert e.value.status == ENONFINITE
    # once the GPU has finished a failing step, the next AdvanceStep raises
    prob.psi.SetData(bad)
    prob.AdvanceStep()
    torch.cuda.synchronize()
    with pytest.raises(_native.GbpropError) as e:
        prob.AdvanceStep()
    assert e.value.status == ENONFINITE
    h.synchronize()                                  # reported once: nothing pending
    _recovers(prob, precision, psi0)


@pytest.mark.parametrize("precision", PRECS)
def test_wait_timeout(precision):
    prob = _problem(precision)
    psi0 = prob.psi.GetDataNumpy().copy()
    h = prob.Propagator.Handle()
    h.debug_set(_native.DEBUG_WAIT_LIMIT, -1)
    try:
        prob.AdvanceStep()
        with pytest.raises(_native.GbpropError) as e:
            h.synchronize()
        assert e.value.status == ETIMEOUT
        # also through the host-buffer entry point, which waits
        host = np.ascontiguousarray(psi0)
        with pytest.raises(_native.GbpropError) as e:
            h.advance_host(host, scalings_for(prob, 1), prob.TimeStep)
        assert e.value.status == ETIMEOUT
    finally:
        h.debug_set(_native.DEBUG_WAIT_LIMIT, 0)
    _recovers(prob, precision, psi0)


@pytest.mark.parametrize("precision", PRECS)
def test_singular_pade_denominator(precision):
    prob = _problem(precision)
    psi0 = prob.psi.GetDataNumpy().copy()
    h = prob.Propagator.Handle()
    h.debug_set(_native.DEBUG_INJECT_LU, 1)
    try:
        prob.AdvanceStep()
        with pytest.raises(_native.GbpropError) as e:
            h.synchronize()
        assert e.value.status == ELU
        # the counters' accessor reports it as well (pAMP's GetOperatorCount path); the failed
        # step left psi undefined (as the reference's throw does), so start from psi0 again
        prob.psi.SetData(psi0)
        prob.AdvanceStep()
        with pytest.raises(_native.GbpropError) as e:
            prob.Propagator.PampWrapper.GetOperatorCount()
        assert e.value.status == ELU
    finally:
        h.debug_set(_native.DEBUG_INJECT_LU, 0)
    _recovers(prob, precision, psi0)


def test_batch_member_failure_reported():
    """A NaN in one problem of a batch is reported by the batch, naming that problem."""
    import torch
    from pyprop_gb300.batch import BatchPropagator, HydrogenProblem
    probs = [HydrogenProblem(lmax=2, nr=30, rmax=20.0, m=6, seed=s) for s in (1, 2, 3)]
    bp = BatchPropagator(probs, autotune=False)
    bp.advance(1)
    bp.synchronize()
    bp.psi[1][0, 3] = float("nan")
    bp.advance(1)
    with pytest.raises(_native.GbpropError) as e:
        bp.synchronize()
    assert e.value.status == ENONFINITE
    assert "problem 1" in str(e.value)
    for p, x in zip(probs, bp.psi):
        x.copy_(torch.as_tensor(p.initial_state()))
    bp.advance(1)
    bp.synchronize()
