"""Batches of uneven independent problems advanced together (one graph launch per
batch step) against the CPU oracle, problem by problem."""
import numpy as np
import pytest

from helpers import rel
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SPECS = [  # lmax, nr, rmax, m, omega, e0, dt
    (2, 20, 30.0, 6, 0.057, 0.05, 0.01),
    (5, 33, 40.0, 8, 0.09, 0.1, 0.02),
    (0, 15, 20.0, 4, 0.05, 0.02, 0.01),
    (3, 41, 60.0, 10, 0.12, 0.08, 0.005),
    (7, 25, 35.0, 12, 0.04, 0.03, 0.01),
]


def _problems():
    from pyprop_gb300.batch import HydrogenProblem
    return [HydrogenProblem(lmax=a, nr=b, rmax=c, m=d, omega=e, e0=f, dt=g, cycles=2, seed=100 + i)
            for i, (a, b, c, d, e, f, g) in enumerate(SPECS)]


def _oracle(prob):
    pots = [dict(kind=orc.ORC_DIAG_BANDNH, data=prob.static, pairs=None, timedep=False),
            dict(kind=orc.ORC_SIMP_BANDNH, data=prob.dipole, pairs=prob.pairs, timedep=True)]
    return orc.Operator(prob.nl, prob.nr, prob.kd, prob.kb, prob.cholesky_band().astype(np.complex128), pots)


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_fp64_vs_oracle(autotune):
    from pyprop_gb300 import _native
    from pyprop_gb300.batch import BatchPropagator
    probs = _problems()
    bp = BatchPropagator(probs, precision=_native.FP64, autotune=autotune)
    psi0 = [p.initial_state() for p in probs]
    bp.advance(3)
    bp.advance(4)          # second call: same graph, new schedule
    for i, p in enumerate(probs):
        want, _ = _oracle(p).advance(psi0[i], p.m, p.dt, bp.scalings(i, 7))
        got = bp.psi[i].cpu().numpy()
        assert rel(got, want) < 1e-12, (i, rel(got, want))


def test_batch_matches_single_problem_path():
    """A problem advanced inside a batch gives the same result as advanced alone."""
    import torch
    from pyprop_gb300 import _native
    from pyprop_gb300.batch import BatchPropagator
    probs = _problems()
    bp = BatchPropagator(probs, precision=_native.FP64, autotune=False)
    bp.advance(5)
    p = probs[3]
    h = p.handle(_native.FP64, torch.cuda.current_stream().cuda_stream)
    d = torch.as_tensor(p.initial_state()).cuda()
    h.advance(d, bp.scalings(3, 5), p.dt)
    assert rel(bp.psi[3].cpu().numpy(), d.cpu().numpy()) < 1e-13


def test_batch_mixed_precision_error_report():
    from pyprop_gb300 import _native
    from pyprop_gb300.batch import BatchPropagator
    probs = _problems()
    bp = BatchPropagator(probs, precision=_native.FP32_MIXED, autotune=False)
    psi0 = [p.initial_state() for p in probs]
    bp.advance(5)
    errs = []
    for i, p in enumerate(probs):
        want, _ = _oracle(p).advance(psi0[i], p.m, p.dt, bp.scalings(i, 5))
        errs.append(rel(bp.psi[i].cpu().numpy().astype(np.complex128), want))
    print("FP32-mixed batch, 5 steps, relative L2 vs FP64 oracle per problem:", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_batch_long_radial_grid(precision):
    """A radial grid long enough that one CTA cannot hold a whole row of the solve: the
    chunking must fit both the FP64 solve and the complex64 basis solve."""
    from pyprop_gb300 import _native
    from pyprop_gb300.batch import BatchPropagator, HydrogenProblem
    # radial sizes around where a whole row stops fitting one CTA (the complex64 solve also
    # stages the FP32 pairs of U~, so its limit is lower than the FP64 solve's)
    probs = [HydrogenProblem(lmax=1, nr=nr, rmax=0.5 * nr, m=8, omega=0.057, e0=0.05, dt=0.005, cycles=2, seed=7 + i)
             for i, nr in enumerate((680, 720, 760, 800, 840, 1400))]
    probs.append(HydrogenProblem(lmax=2, nr=60, rmax=50.0, m=6, omega=0.057, e0=0.05, dt=0.01, cycles=2, seed=3))
    prec = _native.FP64 if precision == "fp64" else _native.FP32_MIXED
    bp = BatchPropagator(probs, precision=prec, autotune=False)
    psi0 = [p.initial_state() for p in probs]
    bp.advance(2)
    for i, p in enumerate(probs):
        want, _ = _oracle(p).advance(psi0[i], p.m, p.dt, bp.scalings(i, 2))
        err = rel(bp.psi[i].cpu().numpy().astype(np.complex128), want)
        assert err < (1e-12 if precision == "fp64" else 1e-5), (i, err)
