"""Bound-state populations and ionisation (pyprop_gb300/observables.py) on the CPU workload: the
hydrogen levels of the consolidated static potential, sum rules in the overlap metric, and their
behaviour under the oracle's unitary propagation."""
import numpy as np

from pyprop_gb300 import observables as ob


def test_bound_state_energies_and_orthonormality(small_problem_cpu):
    states, energies, ls = ob.problem_bound_states(small_problem_cpu)
    S = ob.radial_overlap(small_problem_cpu)
    assert abs(energies[np.argmin(energies)] + 0.5) < 1e-6          # hydrogen 1s
    assert np.all(energies < 0)
    shape = small_problem_cpu.psi.GetData().shape
    for i in range(min(6, len(states))):
        r = ob.report(states[i].reshape(shape), states, S)
        assert abs(r["norm"] - 1.0) < 1e-10
        assert abs(r["populations"][i] - 1.0) < 1e-10             # S-orthonormal set
        assert abs(r["bound"] - 1.0) < 1e-10 and abs(r["ionisation"]) < 1e-10


def test_report_sum_rules_on_the_random_state(small_problem_cpu):
    states, _, _ = ob.problem_bound_states(small_problem_cpu)
    S = ob.radial_overlap(small_problem_cpu)
    psi = small_problem_cpu.psi.GetDataNumpy()                      # seeded, S-normalised
    r = ob.report(psi, states, S)
    assert abs(r["norm"] - 1.0) < 1e-10
    assert np.all(r["populations"] >= 0) and 0.0 <= r["bound"] <= 1.0 + 1e-12
    assert abs(r["bound"] + r["ionisation"] - r["norm"]) < 1e-12


def test_populations_conserved_by_field_free_propagation(small_problem_cpu, small_oracle):
    """Without the field (scaling 0) the bound populations are constants of the motion: exactly
    (to rounding) from the ground state, to the Krylov step's accuracy from the random state, whose
    highest modes carry the approximation error of each step."""
    states, _, _ = ob.problem_bound_states(small_problem_cpu)
    S = ob.radial_overlap(small_problem_cpu)
    psi0 = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    m, dt = small_problem_cpu.Propagator.BasisSize, small_problem_cpu.TimeStep
    psi, _ = small_oracle.advance(psi0, m, dt, [0.0] * 20)
    r0, r1 = ob.report(psi0, states, S), ob.report(psi, states, S)
    assert abs(r1["norm"] - r0["norm"]) < 1e-10
    assert np.max(np.abs(r1["populations"] - r0["populations"])) < 1e-7
    g = states[0].reshape(psi0.shape).astype(np.complex128)
    pg, _ = small_oracle.advance(g, m, dt, [0.0] * 20)
    rg = ob.report(pg, states, S)
    assert abs(rg["populations"][0] - 1.0) < 1e-12 and rg["bound"] - rg["populations"][0] < 1e-12
