"""ctypes front end of the CPU oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
oracle of the GPU path.  Never imported by pyprop_gb300.

Parity status: the reference cannot be built or run here, so this CPU
restatement is pinned by the reference's own known-answer check (TestPade,
core/krylov/pamp/pampwrapper.h:195-217) against scipy, by dense-matrix
numpy/scipy propagation of small cases, by analytic anchors (hydrogen bound
states), and by golden fixtures produced by running the reference's Python
setup modules (tests/golden/make_golden.py).  There are no stored golden
vectors of the propagation itself in the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

ORC_DIAG_BANDNH = 0
ORC_SIMP_BANDNH = 1


class OrcStats(C.Structure):
    _fields_ = [
        ("operator_count", C.c_long),
        ("inner_product_count", C.c_long),
        ("orthogonalization_count", C.c_long),
        ("breakdown_count", C.c_long),
        ("pade_info", C.c_long),
        ("error_estimate", C.c_double),
        ("last_scaling", C.c_int),
        ("last_basis", C.c_int),
    ]


class OrcOperator(C.Structure):
    _fields_ = [
        ("nl", C.c_int), ("nr", C.c_int), ("kb", C.c_int), ("kd", C.c_int),
        ("U", C.c_void_p),
        ("npot", C.c_int),
        ("kind", C.POINTER(C.c_int)),
        ("timedep", C.POINTER(C.c_int)),
        ("npairs", C.POINTER(C.c_int)),
        ("pairs", C.POINTER(C.c_void_p)),
        ("data", C.POINTER(C.c_void_p)),
        ("nfuncs", C.c_int),
    ]


_lib = None


def build():
    """Compile liboracle.so (gcc, OpenMP) if missing or stale."""
    src = os.path.join(HERE, "oracle.c")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        L.orc_zpbtrf_upper.argtypes = [C.c_int, C.c_int, P]
        L.orc_zpbtrf_upper.restype = C.c_int
        L.orc_multiply_potentials.argtypes = [C.POINTER(OrcOperator), P, P, P]
        L.orc_balanced_matvec.argtypes = [C.POINTER(OrcOperator), P, P, P, P]
        L.orc_multiply_sqrt_overlap.argtypes = [C.POINTER(OrcOperator), P]
        L.orc_solve_sqrt_overlap.argtypes = [C.POINTER(OrcOperator), C.c_int, P]
        L.orc_pade_exponential.argtypes = [C.c_int, P, C.c_int, P]
        L.orc_pade_exponential.restype = C.c_int
        L.orc_scaling_pade_exponential.argtypes = [C.c_int, P, C.c_int, P, C.POINTER(C.c_int)]
        L.orc_scaling_pade_exponential.restype = C.c_int
        L.orc_advance.argtypes = [C.POINTER(OrcOperator), P, C.c_int, C.c_double, C.c_double, C.c_int, P, C.c_int,
                                  C.POINTER(OrcStats)]
        L.orc_advance.restype = C.c_int
        L.orc_pamp_once.argtypes = [C.POINTER(OrcOperator), P, C.c_int, C.c_double, C.c_double, P, C.c_int,
                                    P, C.POINTER(OrcStats)]
        L.orc_pamp_once.restype = C.c_int
        L.orc_expokit_advance.argtypes = [C.POINTER(OrcOperator), P, C.c_int, C.c_double, C.c_double, C.c_int, P,
                                          C.c_double, C.c_double, C.POINTER(OrcExpokitStats)]
        L.orc_expokit_advance.restype = C.c_int
        L.orc_arnoldi.argtypes = [C.POINTER(OrcOperator), P, C.c_int, P, C.c_int, P, P, C.POINTER(C.c_double),
                                  C.POINTER(OrcStats)]
        L.orc_arnoldi.restype = C.c_int
        _lib = L
    return _lib


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())


def _p(a):
    return C.c_void_p(a.ctypes.data)


def cholesky_band(S_band_upper, n, kd):
    """zpbtrf 'U' restatement on upper band storage (complex128, (n, kd+1))."""
    a = np.ascontiguousarray(S_band_upper, dtype=np.complex128).copy()
    info = lib().orc_zpbtrf_upper(n, kd, _p(a))
    if info:
        raise np.linalg.LinAlgError("zpbtrf info %d" % info)
    return a


def pade_exponential(A, order=6):
    A = np.ascontiguousarray(A, dtype=np.complex128)
    m = A.shape[0]
    out = np.zeros_like(A)
    info = lib().orc_pade_exponential(m, _p(A), order, _p(out))
    return out, info


def scaling_pade_exponential(A, order=6):
    A = np.ascontiguousarray(A, dtype=np.complex128)
    m = A.shape[0]
    out = np.zeros_like(A)
    s = C.c_int(0)
    info = lib().orc_scaling_pade_exponential(m, _p(A), order, _p(out), C.byref(s))
    return out, info, s.value


class OrcExpokitStats(C.Structure):
    _fields_ = [
        ("substeps", C.c_long),
        ("rejections", C.c_long),
        ("matvecs", C.c_long),
        ("error", C.c_double),
        ("hump", C.c_double),
        ("last_step", C.c_double),
    ]


class Operator:
    """Reference-storage operator: overlap Cholesky factor + consolidated TensorPotential list.

    U_band:     complex128 (nr*(kd+1),) upper band storage
    potentials: list of dict(kind=ORC_DIAG_BANDNH|ORC_SIMP_BANDNH, data=(npairs, (2kb+1)*nr) complex128,
                pairs=(npairs, 2) int32 or None, timedep=False/True or k >= 1: the potential is scaled
                by time function k (True = 1); nfuncs = the largest k)
    Scalings: per step either one value (one time function) or nfuncs values.
    """

    def __init__(self, nl, nr, kd, kb, U_band, potentials):
        self.nl, self.nr, self.kd, self.kb = nl, nr, kd, kb
        self.U = np.ascontiguousarray(U_band, dtype=np.complex128)
        self.pots = []
        for p in potentials:
            data = np.ascontiguousarray(p["data"], dtype=np.complex128)
            pairs = p.get("pairs")
            pairs = np.ascontiguousarray(pairs, dtype=np.int32) if pairs is not None else np.zeros((1, 2), np.int32)
            self.pots.append((int(p["kind"]), int(p["timedep"]), data.shape[0], pairs, data))
        n = len(self.pots)
        self.nfuncs = max([1] + [q[1] for q in self.pots])
        self._kind = (C.c_int * max(n, 1))(*[q[0] for q in self.pots])
        self._td = (C.c_int * max(n, 1))(*[q[1] for q in self.pots])
        self._np = (C.c_int * max(n, 1))(*[q[2] for q in self.pots])
        self._pairs = (C.c_void_p * max(n, 1))(*[q[3].ctypes.data for q in self.pots])
        self._data = (C.c_void_p * max(n, 1))(*[q[4].ctypes.data for q in self.pots])
        self.op = OrcOperator(nl, nr, kb, kd, self.U.ctypes.data, n, self._kind, self._td, self._np,
                              C.cast(self._pairs, C.POINTER(C.c_void_p)), C.cast(self._data, C.POINTER(C.c_void_p)),
                              self.nfuncs)

    @classmethod
    def from_problem(cls, problem):
        """Operator of a pyprop_gb300.Problem (its consolidated potentials and overlap factor)."""
        repr_ = problem.psi.GetRepresentation()
        nl, nr = repr_.GetFullShape()
        kd = repr_.radial.kd
        pots = []
        kb = kd
        nfun = 0
        for p in problem.Propagator.BasePropagator.PotentialList:
            s0, _ = p.GetStorageIds()
            kb = p.GeometryList[1].band_count
            # every time-dependent consolidated potential is scaled by its own time function
            # (TensorPotential.py:98-100): number them in list order
            td = 0
            if p.IsTimeDependent:
                nfun += 1
                td = nfun
            if s0 == "Diag":
                pots.append(dict(kind=ORC_DIAG_BANDNH, data=p.PotentialData, pairs=None, timedep=td))
            elif s0 == "Simp":
                pots.append(dict(kind=ORC_SIMP_BANDNH, data=p.PotentialData, pairs=p.GeometryList[0].GetBasisPairs(),
                                 timedep=td))
            elif s0 == "Ident":
                data = np.repeat(p.PotentialData, nl, axis=0)
                pots.append(dict(kind=ORC_DIAG_BANDNH, data=data, pairs=None, timedep=td))
            else:
                raise NotImplementedError(s0)
        return cls(nl, nr, kd, kb, repr_.radial.cholesky_band().astype(np.complex128), pots)

    def _vec(self, x):
        return np.ascontiguousarray(x, dtype=np.complex128).reshape(self.nl, self.nr).copy()

    def _step_scalings(self, scalings, nsteps=None):
        """(nsteps, nfuncs) contiguous float64: a value per step for one time function, or
        nfuncs values per step; a single value is used for every time function."""
        a = np.asarray(scalings, dtype=np.float64)
        if nsteps is None:                              # one step
            a = a.reshape(-1)
            if a.size == 1:
                a = np.repeat(a, self.nfuncs)
            return np.ascontiguousarray(a.reshape(1, self.nfuncs))
        if a.ndim == 1 and self.nfuncs == 1:
            a = a.reshape(-1, 1)
        return np.ascontiguousarray(a.reshape(nsteps, self.nfuncs))

    def multiply_potentials(self, src, scaling):
        src = self._vec(src)
        dst = np.zeros_like(src)
        s = self._step_scalings(scaling)
        lib().orc_multiply_potentials(C.byref(self.op), _p(s), _p(src), _p(dst))
        return dst

    def balanced_matvec(self, src, scaling):
        src = self._vec(src)
        dst = np.zeros_like(src)
        work = np.zeros_like(src)
        s = self._step_scalings(scaling)
        lib().orc_balanced_matvec(C.byref(self.op), _p(s), _p(src), _p(dst), _p(work))
        return dst

    def multiply_sqrt_overlap(self, psi):
        x = self._vec(psi)
        lib().orc_multiply_sqrt_overlap(C.byref(self.op), _p(x))
        return x

    def solve_sqrt_overlap(self, psi, conj=False):
        x = self._vec(psi)
        lib().orc_solve_sqrt_overlap(C.byref(self.op), int(bool(conj)), _p(x))
        return x

    def advance(self, psi, m, dt, scalings, double_orth=False):
        """len(scalings) PamPropagator steps; returns (psi, stats)."""
        x = self._vec(psi)
        n = np.asarray(scalings).shape[0] if np.ndim(scalings) else 1
        s = self._step_scalings(scalings, n)
        st = OrcStats()
        dt = complex(dt)
        rc = lib().orc_advance(C.byref(self.op), _p(x), int(m), dt.real, dt.imag, n, _p(s),
                               int(bool(double_orth)), C.byref(st))
        if rc:
            raise RuntimeError("oracle Pade LU failed (info %d)" % rc)
        return x, st

    def advance_eigenvector(self, psi, m, dt, scalings, double_orth=False):
        """len(scalings) PamPropagator steps with krylov_exponentiation_method = 1
        (pAMP::EigenvectorExponential, core/krylov/pamp/pamp/pamp.h:567-607): the Arnoldi part in C
        (orc_arnoldi, the same as every step), then A = -i dt H_m, zgeev (numpy.linalg.eig calls
        LAPACK zgeev, the routine the reference calls) for eigenvalues lam and unit right
        eigenvectors W, exp(A) ~ W diag(e^lam) W^H (the reference's formula: W^H, exact for a
        normal A), y = its first column, x = beta0 V^T y (pamp.h:657-662).  Returns (psi, stats)."""
        x = self._vec(psi)
        n = np.asarray(scalings).shape[0] if np.ndim(scalings) else 1
        s = self._step_scalings(scalings, n)
        dt = complex(dt)
        st = OrcStats()
        N = self.nl * self.nr
        V = np.zeros((m, N), dtype=np.complex128)
        H = np.zeros((m, m), dtype=np.complex128)
        for k in range(n):
            lib().orc_multiply_sqrt_overlap(C.byref(self.op), _p(x))
            norm = C.c_double()
            sk = np.ascontiguousarray(s[k])
            lib().orc_arnoldi(C.byref(self.op), _p(x), int(m), _p(sk), int(bool(double_orth)), _p(V), _p(H),
                              C.byref(norm), C.byref(st))
            A = -1j * dt * H
            lam, W = np.linalg.eig(A)
            y = (W * np.exp(lam)[None, :]) @ W[0].conj()
            x = np.ascontiguousarray((norm.value * (y @ V)).reshape(self.nl, self.nr))
            lib().orc_solve_sqrt_overlap(C.byref(self.op), 0, _p(x))
            st.error_estimate = abs(y[m - 1]) ** 2
        return x, st

    def expokit_advance(self, psi, m, dt, scalings, tol, anorm):
        """len(scalings) ExpokitPropagator steps (zgexpv, Krylov dimension m); returns (psi, stats)."""
        x = self._vec(psi)
        n = np.asarray(scalings).shape[0] if np.ndim(scalings) else 1
        s = self._step_scalings(scalings, n)
        st = OrcExpokitStats()
        dt = complex(dt)
        rc = lib().orc_expokit_advance(C.byref(self.op), _p(x), int(m), dt.real, dt.imag, n, _p(s),
                                       float(tol), float(anorm), C.byref(st))
        if rc:
            raise RuntimeError("oracle Expokit failed (%d)" % rc)
        return x, st

    def pamp_once(self, x, m, dt, scaling, double_orth=False):
        """One pAMP call in balanced coordinates; returns (x, scaled Hessenberg, stats)."""
        x = self._vec(x)
        H = np.zeros((m, m), dtype=np.complex128)
        st = OrcStats()
        dt = complex(dt)
        s = self._step_scalings(scaling)
        rc = lib().orc_pamp_once(C.byref(self.op), _p(x), int(m), dt.real, dt.imag, _p(s),
                                 int(bool(double_orth)), _p(H), C.byref(st))
        if rc:
            raise RuntimeError("oracle Pade LU failed (info %d)" % rc)
        return x, H, st

    # dense restatements for cross-checks (numpy) -----------------------------
    def dense_potential(self, scaling):
        """Dense N x N matrix of sum_p s_p V_p in the reference storage semantics."""
        nl, nr, kb = self.nl, self.nr, self.kb
        W = 2 * kb + 1
        H = np.zeros((nl * nr, nl * nr), dtype=np.complex128)
        sc = self._step_scalings(scaling)[0]
        for kind, td, npairs, pairs, data in self.pots:
            s = sc[td - 1] if td else 1.0
            for q in range(npairs):
                row, col = (q, q) if kind == ORC_DIAG_BANDNH else (pairs[q, 0], pairs[q, 1])
                for i in range(nr):
                    for j in range(max(0, i - kb), min(nr, i + kb + 1)):
                        H[row * nr + i, col * nr + j] += s * data[q, j * W + kb + i - j]
        return H

    def dense_U(self):
        nr, kd = self.nr, self.kd
        U = np.zeros((nr, nr), dtype=np.complex128)
        for j in range(nr):
            for i in range(max(0, j - kd), j + 1):
                U[i, j] = self.U[j * (kd + 1) + kd + i - j]
        return np.kron(np.eye(self.nl), U)


# gradient cross-check (dense) --------------------------------------------------
def dense_adjoint_gradient(op, psi0, dt, scalings, states, Sfull=None):
    """Exact discrete gradient of O = sum_b |phi_b^H S psi_T|^2 with respect to the
    step scalings s_n, for the dense step map psi_{n+1} = U^-1 expm(-i dt A(s_n)) U psi_n,
    A(s) = U^-H (H0 + s H1) U^-1 (the map the pAMP step approximates, without Krylov
    truncation; PamPropagator.py:50-57 with the scaling of TensorPotential.py:98-100).

    The reference has no gradient; this dense restatement (scipy expm / expm_frechet,
    co-state y_n = expm(-i dt A_n)^H y_{n+1}, dO/ds_n = 2 Re y_{n+1}^H L_n x_n with L_n the
    Frechet derivative of expm at -i dt A_n in direction -i dt A1) checks the GPU adjoint.
    Returns (O, dO/ds (nsteps,), psi_T)."""
    import scipy.linalg as sl
    U = op.dense_U()
    Ui = np.linalg.inv(U)
    H0 = op.dense_potential(0.0)
    H1 = op.dense_potential(1.0) - H0
    A0 = Ui.conj().T @ H0 @ Ui
    A1 = Ui.conj().T @ H1 @ Ui
    S = U.conj().T @ U if Sfull is None else Sfull
    dt = complex(dt)
    xs = [U @ np.ascontiguousarray(psi0, dtype=np.complex128).ravel()]
    for s in scalings:
        xs.append(sl.expm(-1j * dt * (A0 + s * A1)) @ xs[-1])
    psi_T = Ui @ xs[-1]
    phi = np.asarray(states, dtype=np.complex128)
    amps = phi.conj() @ (S @ psi_T)
    O = float(np.sum(np.abs(amps) ** 2))
    y = U @ (phi.T @ amps)
    g = np.zeros(len(scalings))
    for n in reversed(range(len(scalings))):
        E, L = sl.expm_frechet(-1j * dt * (A0 + scalings[n] * A1), -1j * dt * A1)
        g[n] = 2.0 * np.vdot(y, L @ xs[n]).real
        y = E.conj().T @ y
    return O, g, psi_T.reshape(op.nl, op.nr)
