"""The CPU oracle against known answers: the reference's TestPade matrix, dense
numpy/scipy algebra, and the reference's storage/layout conventions."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

from oracle import oracle as orc


def test_testpade_known_answer():
    # PampWrapper::TestPade (core/krylov/pamp/pampwrapper.h:195-217): A = [[-49, 24], [24, 31]]
    A = np.array([[-49.0, 24.0], [24.0, 31.0]], dtype=np.complex128)
    E, info = orc.pade_exponential(A, 15)
    assert info == 0
    # The unscaled Pade(15) of a matrix of norm ~56 is far from exp; the reference only
    # prints it.  Its known answer is the rational function itself on the eigenvalues.
    def pade15(z):
        c = [1.0]
        for i in range(15):
            c.append(c[-1] * (15 - i) / ((i + 1) * (30 - i)))
        return sum(c[k] * z ** k for k in range(16)) / sum(c[k] * (-z) ** k for k in range(16))
    lam, Q = np.linalg.eigh(A.real)
    assert np.allclose(E, Q @ np.diag(pade15(lam)) @ Q.T, rtol=1e-10)
    iA = 1j * A
    E15, _ = orc.pade_exponential(iA, 15)
    assert np.allclose(E15, Q @ np.diag(pade15(1j * lam)) @ Q.T, rtol=1e-10, atol=1e-12)
    assert np.allclose(E15.conj().T @ E15, np.eye(2), atol=1e-12)      # diagonal Pade of iA is unitary
    ref = sl.expm(iA)
    Es, info, s = orc.scaling_pade_exponential(iA, 6)
    assert info == 0 and s == 6            # ceil(log2(49)) = 6
    assert np.linalg.norm(Es - ref) / np.linalg.norm(ref) < 1e-9


@pytest.mark.parametrize("m", [1, 2, 5, 20, 32])
def test_scaling_pade_vs_scipy(m):
    rng = np.random.default_rng(m)
    H = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    H = (H + H.conj().T) / 2 * 3.0
    A = -1j * 0.3 * H
    E, info, s = orc.scaling_pade_exponential(A, 6)
    assert info == 0
    mx = np.abs(A).max()
    assert s == max(0, int(np.ceil(np.log2(mx))))
    ref = sl.expm(A)
    assert np.linalg.norm(E - ref) / np.linalg.norm(ref) < 1e-6


def test_pade_coefficients_order6_diagonal_form():
    # exp(A) ~ (Q-P)^-1 (Q+P) with P odd, Q even parts of the (6,6) Pade numerator
    A = np.diag([0.3 + 0.1j, -0.2j, 0.05])
    E, info = orc.pade_exponential(A, 6)
    z = np.diag(A)
    c = [1.0]
    for i in range(6):
        c.append(c[-1] * (6 - i) / ((i + 1) * (12 - i)))
    num = sum(c[k] * z ** k for k in range(7))
    den = sum(c[k] * (-z) ** k for k in range(7))
    assert np.allclose(np.diag(E), num / den, rtol=1e-15, atol=0)


def test_zpbtrf_upper_band_storage():
    rng = np.random.default_rng(1)
    n, kd = 30, 4
    M = np.zeros((n, n))
    for d in range(kd + 1):
        v = rng.uniform(-0.2, 0.2, n - d)
        M += np.diag(v, d) + (np.diag(v, -d) if d else 0)
    M += np.eye(n) * 3
    band = np.zeros(n * (kd + 1), dtype=np.complex128)
    for j in range(n):
        for i in range(max(0, j - kd), j + 1):
            band[j * (kd + 1) + kd + i - j] = M[i, j]
    U = orc.cholesky_band(band, n, kd)
    Ud = np.zeros((n, n), dtype=np.complex128)
    for j in range(n):
        for i in range(max(0, j - kd), j + 1):
            Ud[i, j] = U[j * (kd + 1) + kd + i - j]
    assert np.allclose(Ud.conj().T @ Ud, M, atol=1e-13)
    assert np.allclose(Ud, sl.cholesky(M), atol=1e-13)


def test_balanced_matvec_vs_dense(small_problem_cpu, small_oracle):
    op = small_oracle
    psi = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    s = 0.37
    Hd = op.dense_potential(s)
    Ud = op.dense_U()
    Uinv = np.linalg.inv(Ud)
    w = Uinv.conj().T @ (Hd @ (Uinv @ psi.ravel()))
    got = op.balanced_matvec(psi, s).ravel()
    assert np.linalg.norm(got - w) / np.linalg.norm(w) < 1e-13
    # storage consistency (reference storage-consistency check): banded == dense
    got2 = op.multiply_potentials(psi, s).ravel()
    assert np.linalg.norm(got2 - Hd @ psi.ravel()) / np.linalg.norm(got2) < 1e-14


def test_sqrt_overlap_roundtrip(small_problem_cpu, small_oracle):
    psi = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    x = small_oracle.multiply_sqrt_overlap(psi)
    back = small_oracle.solve_sqrt_overlap(x, conj=False)
    assert np.linalg.norm(back - psi) / np.linalg.norm(psi) < 1e-13
    # ||U psi||^2 = psi^H S psi = 1 for the normalised initial state
    assert abs(np.vdot(x, x).real - 1.0) < 1e-12


def _numpy_pamp(A, x, m, dt):
    """Dense numpy restatement of pAMP::PropagateVector (pamp.h:613-669) for cross-checks."""
    N = len(x)
    norm = np.sqrt(np.vdot(x, x).real)
    r = x / norm
    V = np.zeros((m, N), dtype=np.complex128)
    H = np.zeros((m, m), dtype=np.complex128)
    V[0] = r
    r = A @ V[0]
    H[0, 0] = np.vdot(V[0], r)
    r = r - H[0, 0] * V[0]
    for j in range(m - 1):
        beta = np.sqrt(np.vdot(r, r).real)
        if beta < np.sqrt(np.finfo(float).eps):
            break
        V[j + 1] = r / beta
        H[j + 1, j] = beta
        r = A @ V[j + 1]
        h = V[: j + 2].conj() @ r
        r = r - V[: j + 2].T @ h
        H[: j + 2, j + 1] = h
    E, _, _ = orc.scaling_pade_exponential(-1j * dt * H, 6)
    return norm * (V.T @ E[:, 0])


def test_pamp_step_vs_numpy_restatement(small_problem_cpu, small_oracle):
    op = small_oracle
    psi = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    s, dt, m = 0.2, 0.01, 20
    Hd = op.dense_potential(s)
    Ud = op.dense_U()
    Uinv = np.linalg.inv(Ud)
    A = Uinv.conj().T @ Hd @ Uinv
    x = Ud @ psi.ravel()
    want = Uinv @ _numpy_pamp(A, x, m, dt)
    got, st = op.advance(psi, m, dt, [s])
    assert st.operator_count == m
    assert np.linalg.norm(got.ravel() - want) / np.linalg.norm(want) < 1e-12


def test_pamp_small_dt_matches_exact_exponential(small_problem_cpu, small_oracle):
    # for a well-resolved step the Krylov result equals the exact propagator
    op = small_oracle
    psi = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    s, dt, m = 0.0, 1e-5, 20
    Hd = op.dense_potential(s)
    Ud = op.dense_U()
    Uinv = np.linalg.inv(Ud)
    A = Uinv.conj().T @ Hd @ Uinv
    want = Uinv @ (sl.expm(-1j * dt * A) @ (Ud @ psi.ravel()))
    got, _ = op.advance(psi, m, dt, [s])
    assert np.linalg.norm(got.ravel() - want) / np.linalg.norm(want) < 1e-10


def test_unitarity_real_time(small_problem_cpu, small_oracle):
    psi = small_problem_cpu.psi.GetDataNumpy().astype(np.complex128)
    out, _ = small_oracle.advance(psi, 20, 0.01, [0.5] * 5)
    x = small_oracle.multiply_sqrt_overlap(out)
    assert abs(np.vdot(x, x).real - 1.0) < 1e-12


def test_happy_breakdown_eigenvector():
    # a two-level operator: the Krylov space closes after 2 vectors
    nl, nr, kd, kb = 1, 8, 1, 1
    W = 2 * kb + 1
    U = np.zeros(nr * (kd + 1), dtype=np.complex128)
    for j in range(nr):
        U[j * (kd + 1) + kd] = 1.0        # identity overlap
    data = np.zeros((1, W * nr), dtype=np.complex128)
    diag = np.arange(nr, dtype=float)
    for i in range(nr):
        data[0, i * W + kb] = diag[i]
    op = orc.Operator(nl, nr, kd, kb, U, [dict(kind=orc.ORC_DIAG_BANDNH, data=data, pairs=None, timedep=False)])
    psi = np.zeros((1, nr), dtype=np.complex128)
    psi[0, 2] = 1.0
    psi[0, 5] = 1.0
    out, st = op.advance(psi, 6, 0.1, [0.0])
    assert st.breakdown_count == 1 and st.last_basis == 2
    want = psi * np.exp(-1j * 0.1 * diag)
    assert np.allclose(out, want, atol=1e-12)


def test_oracle_reproduces_large_fixture():
    """The oracle built on this host gives the committed states of the benchmarked workload
    (l = 0..63 x 1000, m = 30): 20 steps from the ground state (a smooth map) and one step from
    the seeded random start (a stiff one) within 30x the oracle's sensitivity to a 1e-16 change."""
    import pyprop_gb300 as pp
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_large.npz"))
    conf = pp.Load(os.path.join(os.path.dirname(__file__), "..", "pyprop_gb300", "configs",
                                "hydrogen_velocity_large.ini"))
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    x = prob.psi.GetDataNumpy().astype(np.complex128)
    assert np.linalg.norm(x - g["psi0"]) / np.linalg.norm(x) < 1e-15    # the seeded start (host LAPACK may differ by ulps)
    op = orc.Operator.from_problem(prob)
    m, dt = int(g["m"]), complex(g["dt"])
    psi, _ = op.advance(g["gs0"], m, dt, g["scalings"][:20])
    assert np.linalg.norm(psi - g["gs20"]) / np.linalg.norm(g["gs20"]) < 1e-13
    psi, _ = op.advance(g["psi0"], m, dt, g["scalings"][:1])
    assert np.linalg.norm(psi - g["rand1"]) / np.linalg.norm(g["rand1"]) < 30 * float(g["sens1"])
