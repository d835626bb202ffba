"""Final-state observables of the hydrogen examples: bound-state populations and
ionisation probability.

The field-free bound states are the eigenvectors with E < 0 of the static
(time-independent, angular-diagonal) TensorPotentials in the B-spline overlap metric,
one generalized eigenproblem H0_l c = E S c per angular row l; the population of state b
is |<phi_b|S|psi>|^2 and the ionisation probability 1 - sum_b |<phi_b|S|psi>|^2 (for a
normalised psi).  This follows the analysis of the reference's hydrogen example
(examples/tensor/helium_stabilization_sae/analysis.py:92-160, 344-375), restated.
"""
from __future__ import annotations

import math

import numpy as np

from .tensorpotential import bandnh_to_dense


def _dense_from_diagonals(D, kd, n):
    S = np.zeros((n, n))
    for d in range(-kd, kd + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        S[i, i + d] = D[kd + d, i]
    return S


def bound_states(nl, nr, kb, S, static_rows, emax=0.0, lmax_states=None):
    """Bound eigenstates of the angular-diagonal static operator.

    S: dense radial overlap (nr, nr); static_rows[l]: BandNH data of row l (complex, real-valued).
    Returns (states (nb, nl*nr) complex, S-normalised; energies (nb,); l of each state (nb,))."""
    import scipy.linalg as sl
    states, energies, ls = [], [], []
    last = nl if lmax_states is None else min(nl, lmax_states + 1)
    for l in range(last):
        H = bandnh_to_dense(np.asarray(static_rows[l]), nr, kb).real
        H = 0.5 * (H + H.T)
        e, v = sl.eigh(H, S)
        for j in np.where(e < emax)[0]:
            phi = np.zeros((nl, nr), dtype=np.complex128)
            phi[l] = v[:, j] / math.sqrt(v[:, j] @ S @ v[:, j])
            states.append(phi.ravel())
            energies.append(e[j])
            ls.append(l)
    return np.array(states), np.array(energies), np.array(ls)


def _symmetric_bands(v, nr, kb):
    """Diagonal-major symmetric band B[d, i] = (H(i, i+d-kb) + H(i+d-kb, i)) / 2 of a row's
    BandNH data (real part; the static operators are real)."""
    W = 2 * kb + 1
    v = np.asarray(v).real
    B = np.zeros((W, nr))
    for d in range(W):
        off = d - kb
        i = np.arange(max(0, -off), min(nr, nr - off))
        j = i + off
        B[d, i] = v[j * W + kb + i - j]
    Bs = np.zeros_like(B)
    for d in range(W):
        off = d - kb
        i = np.arange(max(0, -off), min(nr, nr - off))
        Bs[d, i] = 0.5 * (B[d, i] + B[2 * kb - d, i + off])
    return Bs


def bound_states_device(nl, nr, kb, Sdiag, static_rows, emax=0.0, lmax_states=None, max_states=64, device="cuda"):
    """bound_states() on the GPU (gbprop_bound_states: inertia counts of banded LDL^T
    factorisations, bisection, inverse iteration; one thread per state), from the banded
    operators directly -- no dense eigenproblem.  Sdiag: overlap diagonals D[kb + d, i] =
    S(i, i+d).  Same return values as bound_states() (numpy)."""
    import torch

    from . import _native
    last = nl if lmax_states is None else min(nl, lmax_states + 1)
    Sdiag = np.ascontiguousarray(np.asarray(Sdiag, dtype=np.float64))
    if Sdiag.shape != (2 * kb + 1, nr):
        raise ValueError("overlap diagonals must be (2kb+1, nr) = %s, got %s" % ((2 * kb + 1, nr), Sdiag.shape))
    Hb = np.stack([_symmetric_bands(static_rows[l], nr, kb) for l in range(last)])
    counts, energies, vecs = _native.bound_states(torch.as_tensor(Hb, device=device),
                                                  torch.as_tensor(Sdiag, device=device), emax, max_states)
    vecs = vecs.cpu().numpy()
    states, es, ls = [], [], []
    for l in range(last):
        for k in range(min(int(counts[l]), max_states)):
            phi = np.zeros((nl, nr), dtype=np.complex128)
            phi[l] = vecs[l, k]
            states.append(phi.ravel())
            es.append(energies[l, k])
            ls.append(l)
    return np.array(states), np.array(es), np.array(ls)


def _solver(solver):
    """"auto": the GPU eigensolver when a CUDA device is present, else the host's."""
    if solver != "auto":
        return solver
    try:
        import torch
        return "gpu" if torch.cuda.is_available() else "host"
    except ImportError:
        return "host"


def problem_bound_states(problem, emax=0.0, lmax_states=None, solver="auto"):
    """bound_states() of a pyprop_gb300.Problem (its consolidated static Diag potentials);
    solver "gpu": bound_states_device(), "host": scipy per row, "auto": the GPU when present."""
    solver = _solver(solver)
    repr_ = problem.psi.GetRepresentation()
    nl, nr = repr_.GetFullShape()
    rad = repr_.radial
    S = _dense_from_diagonals(rad.overlap_diagonals(), rad.kd, nr)
    static = None
    kb = rad.kd
    for p in problem.Propagator.BasePropagator.PotentialList:
        if p.IsTimeDependent:
            continue
        s0, _ = p.GetStorageIds()
        kb = p.GeometryList[1].band_count
        if s0 == "Diag":
            rows = np.asarray(p.PotentialData)
        elif s0 == "Ident":
            rows = np.repeat(np.asarray(p.PotentialData), nl, axis=0)
        else:
            raise NotImplementedError("bound states need angular-diagonal static potentials (got %s)" % s0)
        static = rows if static is None else static + rows
    if solver == "gpu":
        return bound_states_device(nl, nr, kb, rad.overlap_diagonals(), static, emax, lmax_states)
    return bound_states(nl, nr, kb, S, static, emax, lmax_states)


def hydrogen_bound_states(hp, emax=0.0, lmax_states=None, solver="auto"):
    """bound_states() of a batch.HydrogenProblem; solver as problem_bound_states()."""
    if _solver(solver) == "gpu":
        return bound_states_device(hp.nl, hp.nr, hp.kb, hp.Sdiag, hp.static, emax, lmax_states)
    S = _dense_from_diagonals(hp.Sdiag, hp.kd, hp.nr)
    return bound_states(hp.nl, hp.nr, hp.kb, S, hp.static, emax, lmax_states)


def populations(psi, states, S):
    """|<phi_b|S|psi>|^2 per state; psi (nl, nr) numpy, S dense radial overlap."""
    psi = np.asarray(psi, dtype=np.complex128)
    Spsi = (psi @ S.T).ravel()
    amps = np.conj(states) @ Spsi
    return np.abs(amps) ** 2


def overlap_norm2(psi, S):
    psi = np.asarray(psi, dtype=np.complex128)
    return float(np.real(np.sum(np.conj(psi) * (psi @ S.T))))


def report(psi, states, S):
    """Populations per bound state, their sum and the ionisation probability 1 - sum."""
    pops = populations(psi, states, S)
    norm = overlap_norm2(psi, S)
    return {"populations": pops, "bound": float(pops.sum()), "ionisation": float(norm - pops.sum()), "norm": norm}


def radial_overlap(problem):
    """Dense radial overlap matrix of a Problem."""
    rad = problem.psi.GetRepresentation().radial
    return _dense_from_diagonals(rad.overlap_diagonals(), rad.kd, rad.count)


class DevicePopulations:
    """Bound-state populations and ionisation of DEVICE wavefunctions, evaluated on the GPU
    (the per-state projections of analysis.py:344-375 restated): the bra rows (S phi_b) are
    formed once and kept on the device; every evaluation is one block inner product per 45
    states (gbprop_block_inner_product, the Arnoldi step's inner-product kernel) and the
    overlap-metric norm from the handle (gbprop_inner_product).  The eigenproblems giving the
    states are solved once, at set-up, on the host.

    states: (nb, nl*nr) S-normalised bound states (bound_states()); S: dense radial overlap;
    handle: the propagator's libgbprop handle (for ||psi||_S)."""

    def __init__(self, states, S, handle, device="cuda"):
        import torch
        states = np.asarray(states, dtype=np.complex128)
        nb = states.shape[0]
        nr = S.shape[0]
        nl = states.shape[1] // nr
        bra = (states.reshape(nb, nl, nr) @ S.T).reshape(nb, -1)        # (S phi_b) rows, S real symmetric
        self.bra = torch.as_tensor(np.ascontiguousarray(bra)).to(device)
        self.handle = handle
        self.nb = nb

    def populations(self, psi):
        """|<phi_b|S|psi>|^2 (device float64 tensor, one per state)."""
        import torch
        from . import _native
        w = psi.reshape(-1)
        if w.dtype != torch.complex128:
            w = w.to(torch.complex128)
        out = []
        for k0 in range(0, self.nb, 45):
            r = _native.block_inner_product(self.bra[k0:k0 + 45], w)
            out.append(r[0::2] ** 2 + r[1::2] ** 2)
        return torch.cat(out)

    def report(self, psi):
        """As report(): populations, their sum ('bound'), norm - bound ('ionisation'), the norm."""
        pops = self.populations(psi).cpu().numpy()
        norm = self.handle.inner_product(psi, psi).real
        return {"populations": pops, "bound": float(pops.sum()), "ionisation": float(norm - pops.sum()), "norm": norm}
