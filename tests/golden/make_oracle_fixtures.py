"""Oracle outputs for the CPU-runnable workload (hydrogen, l=0..9 x 106 B-splines,
m=20, dt=0.01, 500 steps), saved so that GPU parity tests need not re-run the
oracle.  Usage: python tests/golden/make_oracle_fixtures.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import pyprop_gb300 as pp  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = os.path.join(HERE, "oracle_small.npz")


def main():
    conf = pp.Load(os.path.join(ROOT, "pyprop_gb300", "configs", "hydrogen_velocity_small.ini"))
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    op = orc.Operator.from_problem(prob)
    bp = prob.Propagator.BasePropagator
    nsteps = 500
    times, t = [], prob.PropagatedTime
    for _ in range(nsteps):
        times.append(t)
        t = prob._next_time(t)
    scal = np.array([bp._scaling(x) for x in times])
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    m = prob.Propagator.BasisSize
    t0 = time.time()
    psi20, st20 = op.advance(psi0, m, prob.TimeStep, scal[:20])
    psi500, st = op.advance(psi20, m, prob.TimeStep, scal[20:])
    print("oracle 500 steps: %.1f s" % (time.time() - t0))
    np.savez_compressed(OUT, psi0=psi0, scalings=scal, psi20=psi20, psi500=psi500, m=m,
                        dt=np.array(prob.TimeStep), ops=st20.operator_count + st.operator_count)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
