"""Oracle outputs saved so that GPU parity tests compare against fixed vectors as well as
against the oracle re-run on the GPU host.  Usage:

    python tests/golden/make_oracle_fixtures.py [small] [large] [batch]

small  hydrogen, l=0..9 x 106 B-splines, m=20, dt=0.01: states after 20 and 500 steps from the
       configured seeded random start (oracle_small.npz)
large  hydrogen at scale, l=0..63 x 1000 B-splines, m=30, dt=0.005 (the benchmarked workload),
       oracle_large.npz:
         rand1, rand2   states after 1 and 2 steps from the configured seeded random start, and
         sens1, sens2   the oracle's own sensitivity there: the relative change of those states
                        for a seeded 1e-16 relative change of the start.  Random B-spline
                        coefficients fill the stiffest modes (||dt H_m|| ~ 2^17), where the
                        unconverged m = 30 Krylov step amplifies rounding ~1e4-fold per step: after
                        5 steps the state depends on the summation order at the 10% level, for the
                        reference's algorithm as for any restatement of it.
         gs0            the hydrogen ground state (1s) in this basis, and
         gs20/200/2000  the states after 20, 200 and 2000 steps from it (the whole pulse), with
         gs_sens*       the oracle's sensitivity along that run: the map is smooth while the
                        field is weak (3e-15 after 20 steps); as the pulse moves population into
                        the stiff modes it amplifies rounding too (2e-10 after 50 steps, 1e-9
                        after 100)
batch  the largest problem size of the 256-problem batch, l=0..64 x 1500 B-splines, r_max=400,
       m=32, dt=0.01, field from t = 100 (oracle_batch_large.npz): rand1/sens1 from the seeded
       random start; gs1, gs20 and gs_sens1, gs_sens20 from the ground state gs0
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

CONFIGS = os.path.join(ROOT, "pyprop_gb300", "configs")


def _scalings(prob, nsteps):
    bp = prob.Propagator.BasePropagator
    times, t = [], prob.PropagatedTime
    for _ in range(nsteps):
        times.append(t)
        t = prob._next_time(t)
    return np.array([bp._scaling(x) for x in times])


def _load(ini):
    conf = pp.Load(os.path.join(CONFIGS, ini))
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    return prob, orc.Operator.from_problem(prob)


def _run(op, psi, m, dt, scal, checkpoints, tag, label):
    out, done = {}, 0
    t0 = time.time()
    st = None
    for c in checkpoints:
        psi, st = op.advance(psi, m, dt, scal[done:c])
        out["%s%d" % (tag, c)] = psi.copy()
        done = c
        print("  %s: %d steps (%.1f s)" % (label, c, time.time() - t0), flush=True)
    return out, st


def _sensitivity(op, psi0, m, dt, scal, checkpoints, seed=3):
    """Relative change of the states for a seeded 1e-16 relative change of the start."""
    rng = np.random.default_rng(seed)
    pert = psi0 * (1 + 1e-16 * rng.standard_normal(psi0.shape))
    a, _ = _run(op, psi0.copy(), m, dt, scal, checkpoints, "x", "sensitivity (start)")
    b, _ = _run(op, pert, m, dt, scal, checkpoints, "x", "sensitivity (perturbed start)")
    return {"sens%d" % c: np.linalg.norm(a["x%d" % c] - b["x%d" % c]) / np.linalg.norm(a["x%d" % c])
            for c in checkpoints}


def small():
    prob, op = _load("hydrogen_velocity_small.ini")
    scal = _scalings(prob, 500)
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    m = prob.Propagator.BasisSize
    out, st = _run(op, psi0, m, prob.TimeStep, scal, [20, 500], "psi", "small")
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), psi0=psi0, scalings=scal, m=m,
                        dt=np.array(prob.TimeStep), **out)


def large():
    from pyprop_gb300 import observables as ob
    prob, op = _load("hydrogen_velocity_large.ini")
    scal = _scalings(prob, 2000)
    psi0 = prob.psi.GetDataNumpy().astype(np.complex128)
    m, dt = prob.Propagator.BasisSize, prob.TimeStep
    rand, st_r = _run(op, psi0, m, dt, scal, [1, 2], "rand", "large, random start")
    sens = _sensitivity(op, psi0, m, dt, scal, [1, 2])
    states, _, _ = ob.problem_bound_states(prob, lmax_states=0)
    gs0 = states[0].reshape(psi0.shape).astype(np.complex128)
    gs, st_g = _run(op, gs0, m, dt, scal, [20, 200, 2000], "gs", "large, ground-state start")
    gsens = {"gs_" + k: v for k, v in _sensitivity(op, gs0, m, dt, scal, [20, 200, 2000]).items()}
    np.savez_compressed(os.path.join(HERE, "oracle_large.npz"), psi0=psi0, scalings=scal, m=m, dt=np.array(dt),
                        gs0=gs0, rand_scaling_order=st_r.last_scaling, gs_scaling_order=st_g.last_scaling,
                        **rand, **sens, **gs, **gsens)


def batch():
    from pyprop_gb300 import observables as ob
    from pyprop_gb300.batch import HydrogenProblem
    p = HydrogenProblem(lmax=64, nr=1500, rmax=400.0, m=32, dt=0.01, omega=0.04, e0=0.1, seed=20261206)
    pots = [dict(kind=orc.ORC_DIAG_BANDNH, data=p.static, pairs=None, timedep=False),
            dict(kind=orc.ORC_SIMP_BANDNH, data=p.dipole, pairs=p.pairs, timedep=True)]
    op = orc.Operator(p.nl, p.nr, p.kd, p.kb, p.cholesky_band().astype(np.complex128), pots)
    nsteps = 20
    scal = np.array([p.field(k * p.dt.real + 100.0) for k in range(nsteps)])
    psi0 = p.initial_state()
    rand, _ = _run(op, psi0, p.m, p.dt, scal, [1], "rand", "batch-sized, random start")
    sens = _sensitivity(op, psi0, p.m, p.dt, scal, [1])
    states, _, _ = ob.hydrogen_bound_states(p, lmax_states=0)
    gs0 = states[0].reshape(psi0.shape).astype(np.complex128)
    gs, st = _run(op, gs0, p.m, p.dt, scal, [1, nsteps], "gs", "batch-sized, ground-state start")
    gsens = {"gs_" + k: v for k, v in _sensitivity(op, gs0, p.m, p.dt, scal, [1, nsteps]).items()}
    np.savez_compressed(os.path.join(HERE, "oracle_batch_large.npz"), psi0=psi0, scalings=scal, m=p.m,
                        dt=np.array(p.dt), gs0=gs0, gs_scaling_order=st.last_scaling, **rand, **sens, **gs, **gsens)


if __name__ == "__main__":
    orc.set_threads(os.cpu_count() or 1)
    which = sys.argv[1:] or ["small", "large", "batch"]
    for w in which:
        globals()[w]()
        print("wrote", w, flush=True)
