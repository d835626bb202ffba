"""Field-free bound states on the GPU (gbprop_bound_states: banded LDL^T inertia counts,
bisection, inverse iteration) against the host's dense generalized eigensolver (scipy eigh per
angular row, the analysis of examples/tensor/helium_stabilization_sae/analysis.py:92-160)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare(host, gpu, S, nr):
    (sh, eh, lh), (sg, eg, lg) = host, gpu
    assert len(eh) == len(eg) and np.array_equal(lh, lg)
    assert np.max(np.abs(eg - eh)) < 1e-12 * max(1.0, np.max(np.abs(eh)))
    # vectors: sign-free overlap in the S metric, per state (row by row)
    worst = 0.0
    for a, b, l in zip(sh, sg, lh):
        ra = a.reshape(-1, nr)[l]
        rb = b.reshape(-1, nr)[l]
        ov = abs(np.real(np.conj(ra) @ S @ rb))
        worst = max(worst, abs(ov - 1.0))
        assert abs(ov - 1.0) < 1e-12, (l, ov)
    print("\nmax |1 - |<phi_host|S|phi_gpu>|| = %.2e" % worst)
    return np.max(np.abs(eg - eh))


def test_bound_states_small_workload_vs_host():
    import pyprop_gb300 as pp
    from pyprop_gb300 import observables as ob
    from helpers import make_problem
    prob = make_problem(maxl=9, xsize=103, m=20, dt=0.01)
    host = ob.problem_bound_states(prob, solver="host")
    gpu = ob.problem_bound_states(prob, solver="gpu")
    S = ob.radial_overlap(prob)
    err = _compare(host, gpu, S, S.shape[0])
    print("\n%d bound states, max |E_gpu - E_host| %.2e, lowest %.15f" % (len(host[1]), err, gpu[1].min()))


def test_bound_states_hydrogen_problem_vs_host_and_hydrogenic_levels():
    from pyprop_gb300 import observables as ob
    from pyprop_gb300.batch import HydrogenProblem
    hp = HydrogenProblem(lmax=12, nr=300, rmax=150.0, m=16, dt=0.01, seed=5)
    host = ob.hydrogen_bound_states(hp, solver="host")
    gpu = ob.hydrogen_bound_states(hp, solver="gpu")
    from pyprop_gb300.observables import _dense_from_diagonals
    S = _dense_from_diagonals(hp.Sdiag, hp.kd, hp.nr)
    err = _compare(host, gpu, S, hp.nr)
    # eigen-residuals ||(H_l - E S) x|| / (||H_l|| ||x||) of both solvers' vectors
    from pyprop_gb300.tensorpotential import bandnh_to_dense
    res = {}
    for name, (st, en, ll) in (("host", host), ("gpu", gpu)):
        worst = 0.0
        for x, E, lq in zip(st, en, ll):
            H = bandnh_to_dense(np.asarray(hp.static[lq]), hp.nr, hp.kb).real
            H = 0.5 * (H + H.T)
            v = np.real(x.reshape(-1, hp.nr)[lq])
            r = H @ v - E * (S @ v)
            worst = max(worst, np.linalg.norm(r) / (np.linalg.norm(H, 2) * np.linalg.norm(v)))
        res[name] = worst
    print("\nmax relative eigen-residual: host %.2e, gpu %.2e" % (res["host"], res["gpu"]))
    assert res["gpu"] < 1e-14
    e, l = gpu[1], gpu[2]
    # the lowest levels of each l are hydrogenic: E = -1 / (2 n^2), n = l + 1, l + 2, ...
    for ll in range(3):
        el = np.sort(e[l == ll])
        for j in range(3):
            n = ll + 1 + j
            assert abs(el[j] + 0.5 / n ** 2) < 1e-6 * (0.5 / n ** 2), (ll, j, el[j])
    print("\n%d bound states, max |E_gpu - E_host| %.2e" % (len(e), err))


def test_bound_states_at_batch_scale():
    """The largest batch size (l = 0..64 x 1500 B-splines, r_max 400): every row's count equals the
    number of negative energies found, the lowest level of each l is hydrogenic."""
    from pyprop_gb300 import observables as ob
    from pyprop_gb300.batch import HydrogenProblem
    hp = HydrogenProblem(lmax=64, nr=1500, rmax=400.0, m=32, dt=0.01, seed=6, setup="gpu")
    t0 = time.perf_counter()
    states, e, l = ob.hydrogen_bound_states(hp, solver="gpu")
    dt = time.perf_counter() - t0
    print("\n%d bound states of 65 rows x 1500 in %.2f s" % (len(e), dt))
    assert np.all(e < 0) and len(e) > 65
    for ll in (0, 1, 10):
        assert abs(np.sort(e[l == ll])[0] + 0.5 / (ll + 1) ** 2) < 1e-6 * (0.5 / (ll + 1) ** 2)
