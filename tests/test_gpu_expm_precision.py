"""The Hessenberg exponentials on the Hessenberg matrix of a real step (m = 30): the FP64 Pade
scaling-and-squaring (pamp.h:480-564), the double-float Pade of the FP32-mixed path and the
eigenvector form (pamp.h:567-607), each against scipy's expm of the same -i dt H (column 0),
through gbprop_debug_expm."""
import numpy as np
import pytest

from helpers import make_problem, rel
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [0.01, 0.05])
def test_exponentials_vs_scipy(dt):
    import scipy.linalg as sla
    prob = make_problem(maxl=7, xsize=60, m=30, dt=dt)
    prob.AdvanceStep()
    h = prob.Propagator.Handle()
    H = 1j * h.hessenberg() / dt
    want = sla.expm((-1j * dt) * H)[:, 0]
    y64, s64 = h.debug_expm(H, dt, 0)
    ydf, sdf = h.debug_expm(H, dt, 1)
    yeig, _ = h.debug_expm(H, dt, 2)
    e64, edf, eeig = rel(y64, want), rel(ydf, want), rel(yeig, want)
    print("\ndt %.3g, ||dt H||_inf %.3g, scaling order %d: FP64 Pade %.2e | double-float Pade %.2e | "
          "eigenvector %.2e" % (dt, dt * np.abs(H).sum(axis=1).max(), s64, e64, edf, eeig))
    assert s64 == sdf and s64 > 0
    # the same algorithm on the CPU (the oracle's ScalingPadeExponential, pamp.h:430-564)
    A = (-1j * dt) * H
    ref, info, s_ref = orc.scaling_pade_exponential(A)
    assert info == 0
    e_orc = rel(y64, ref[:, 0])
    print("FP64 Pade vs the oracle's: %.2e (scaling orders %d, %d)" % (e_orc, s64, s_ref))
    assert s64 == s_ref
    # s squarings double the relative error s times; bounds of a few units of each arithmetic's
    # rounding (FP64 1.1e-16, double-float ~2^-48) times 2^s
    assert e_orc < 2.0 ** s64 * 1e-15 + 1e-14
    assert e64 < 2.0 ** s64 * 4e-15 + 1e-13      # Pade(6) after scaling, against scipy's Pade(13)
    assert edf < 2.0 ** s64 * 3e-14 + 1e-12
    assert eeig < 1e-11
