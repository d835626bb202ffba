"""Gradients of final-state observables with respect to field samples.

The reference has no adjoint; this module adds one on top of the same GPU
propagation step.  The control is a piecewise-linear time function
s(t) = sum_k c_k phi_k(t) (hat functions on a uniform grid over [0, T]) that
scales the time-dependent TensorPotential (the velocity-gauge dipole term), so
the step map of step n is

    psi_{n+1} = F_n(psi_n; s_n),   F_n = U^-1 exp(-i dt (A0 + s_n A1)) U,
    s_n = s(t_n) at the step start (TensorPotential.py:98-100).

Hand-written discrete adjoint (backward-in-time Krylov propagation of the
co-state), with O = sum_b |<phi_b|S|psi_T>|^2 for a set of bound states b:
  * terminal co-state gamma_T = sum_b phi_b <phi_b|S|psi_T> (physical form of
    U^-H dO/dpsi-bar, so that dO = 2 Re gamma^H S dpsi);
  * gamma_n = F_n^H-like step: exp(+i dt A_n) in balanced coordinates, i.e. the
    same pAMP step with dt -> -dt and the same s_n;
  * dO/ds_n = 2 Re gamma_{n+1}^H S (d psi_{n+1}/d s_n), where the derivative of
    the exponential is taken exactly from the block-triangular operator
        exp(-i dt [[A, A1], [0, A]]) [0; x] = [d(exp(-i dt A) x)/ds; exp(-i dt A) x],
    which runs on the same kernels as a problem with 2*nl angular rows;
  * dO/dc_k = sum_n phi_k(t_n) dO/ds_n.
Forward states are checkpointed every `checkpoint` steps and the steps in
between are recomputed during the backward sweep.

`ObservableFunction` wraps this as a torch.autograd.Function of the samples.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native


def hat_weights(times, T, nsamples):
    """phi_k(t_n): piecewise-linear interpolation weights of `nsamples` uniform samples over [0, T]."""
    W = np.zeros((len(times), nsamples))
    for n, t in enumerate(times):
        if not (0 <= t <= T):
            continue
        x = t / T * (nsamples - 1)
        k = min(int(math.floor(x)), nsamples - 2)
        w = x - k
        W[n, k] += 1.0 - w
        W[n, k + 1] += w
    return W


def bound_states(problem, emax=0.0, lmax_states=None, solver="auto"):
    """Bound eigenstates (E < emax) of a batch.HydrogenProblem's field-free Hamiltonian, per l,
    S-normalised physical coefficient vectors (observables.hydrogen_bound_states; solver "gpu" or
    "auto" with a CUDA device: the banded GPU eigensolver)."""
    from .observables import hydrogen_bound_states
    return hydrogen_bound_states(problem, emax, lmax_states, solver=solver)


class AugmentedOperator:
    """The problem with 2*nl angular rows whose step gives [dF/ds psi; F psi] from [0; psi]:
    rows 0..nl-1 carry A u + A1 v, rows nl..2nl-1 carry A v (A = A0 + s A1)."""

    @staticmethod
    def potentials(problem):
        nl = problem.nl
        static, dip, pairs = problem.static, problem.dipole, problem.pairs
        pr = np.asarray(pairs, dtype=np.int32)
        p_dip = np.concatenate([pr, pr + nl]).astype(np.int32)
        p_cpl = np.stack([pr[:, 0], pr[:, 1] + nl], 1).astype(np.int32)   # (dst u-row, src v-row)
        return [(_native.STORAGE_DIAG, None, np.concatenate([static, static]), False),
                (_native.STORAGE_SIMP, p_dip, np.concatenate([dip, dip]), True),
                (_native.STORAGE_SIMP, p_cpl, dip, False)]

    @staticmethod
    def handle(problem, m, precision=_native.FP64, stream=0):
        h = _native.Handle(2 * problem.nl, problem.nr, precision, m, 0, False, stream)
        h.set_overlap(problem.kd, problem.cholesky_band())
        for storage, pairs, data, td in AugmentedOperator.potentials(problem):
            h.add_potential(storage, pairs, problem.kb, data, td)
        h.finalize()
        return h


class AdjointPropagator:
    """Forward propagation with checkpoints, and the adjoint gradient of
    O = sum_b |<phi_b|S|psi_T>|^2 with respect to the field samples."""

    def __init__(self, problem, nsteps, nsamples, checkpoint=50, precision=_native.FP64, m_aug=None,
                 device="cuda"):
        import torch
        self.torch = torch
        self.problem = problem
        self.nsteps = int(nsteps)
        self.nsamples = int(nsamples)
        self.checkpoint = int(checkpoint)
        self.precision = precision
        self.device = device
        self.dt = complex(problem.dt)
        self.T = self.nsteps * self.dt.real
        self.times = np.array([n * self.dt.real for n in range(self.nsteps)])
        self.W = hat_weights(self.times, self.T, self.nsamples)
        stream = torch.cuda.current_stream().cuda_stream
        self.h = problem.handle(precision, stream)
        self.m_aug = int(m_aug or min(2 * problem.m, 45))
        self.h_aug = AugmentedOperator.handle(problem, self.m_aug, precision, stream)
        self.cdt = torch.complex128 if precision == _native.FP64 else torch.complex64
        D = torch.as_tensor(problem.Sdiag, dtype=torch.float64, device=device)
        self._S = D

    # -- helpers ----------------------------------------------------------------
    def _apply_S(self, x):
        torch = self.torch
        kd, nr = self.problem.kd, self.problem.nr
        xd = x.to(torch.complex128)
        out = torch.zeros_like(xd)
        for d in range(-kd, kd + 1):
            lo, hi = max(0, -d), min(nr, nr - d)
            out[:, lo:hi] += self._S[kd + d, lo:hi] * xd[:, lo + d:hi + d]
        return out

    def scalings(self, samples):
        return self.W @ np.asarray(samples, dtype=np.float64)

    # -- forward ----------------------------------------------------------------
    def forward(self, psi0, samples, keep=True):
        """Propagate psi0 (numpy (nl, nr)) over nsteps; returns the final state tensor.
        Checkpoints every `checkpoint` steps are kept for the backward sweep."""
        torch = self.torch
        s = self.scalings(samples)
        psi = torch.as_tensor(np.ascontiguousarray(psi0)).to(self.device, self.cdt).clone()
        # a new dict per call: a caller holding the previous call's tape keeps its checkpoints
        self._ckpt = {}
        self._s = s
        for n0 in range(0, self.nsteps, self.checkpoint):
            if keep:
                self._ckpt[n0] = psi.clone()
            n1 = min(self.nsteps, n0 + self.checkpoint)
            self.h.advance(psi, s[n0:n1], self.dt)
        return psi

    # -- observables ----------------------------------------------------------------
    def populations(self, psi, states):
        """|<phi_b|S|psi>|^2 for every row of `states` (numpy (nb, N))."""
        torch = self.torch
        phi = torch.as_tensor(states).to(self.device, torch.complex128)
        Spsi = self._apply_S(psi).reshape(-1)
        amps = torch.conj(phi) @ Spsi
        return (amps.abs() ** 2).cpu().numpy(), amps

    def observable(self, psi, states):
        return float(self.populations(psi, states)[0].sum())

    # -- adjoint ----------------------------------------------------------------
    def tape(self):
        """The checkpoints and field values of the last forward(keep=True) call; pass it to
        gradient() to differentiate that call after later forward calls."""
        return (self._ckpt, self._s)

    def gradient(self, psi_T, states, tape=None):
        """dO/dc_k for O = sum_b |<phi_b|S|psi_T>|^2, for the forward call whose tape() is given
        (default: the last forward(keep=True) call)."""
        torch = self.torch
        ckpt, svals = tape if tape is not None else self.tape()
        nl, nr = self.problem.nl, self.problem.nr
        phi = torch.as_tensor(states).to(self.device, torch.complex128)
        Spsi = self._apply_S(psi_T).reshape(-1)
        amps = torch.conj(phi) @ Spsi
        gamma = (phi.T @ amps).reshape(nl, nr).to(self.cdt)        # terminal co-state (physical form)
        dOds = torch.zeros(self.nsteps, dtype=torch.float64, device=self.device)
        aug = torch.zeros((2 * nl, nr), dtype=self.cdt, device=self.device)
        for n0 in reversed(range(0, self.nsteps, self.checkpoint)):
            n1 = min(self.nsteps, n0 + self.checkpoint)
            # recompute the forward states of this segment from its checkpoint
            states_seg = [ckpt[n0].clone()]
            psi = ckpt[n0].clone()
            for n in range(n0, n1 - 1):
                self.h.advance(psi, svals[n:n + 1], self.dt)
                states_seg.append(psi.clone())
            for n in reversed(range(n0, n1)):
                psi_n = states_seg[n - n0]
                aug.zero_()
                aug[nl:] = psi_n
                self.h_aug.advance(aug, svals[n:n + 1], self.dt)
                dpsi = aug[:nl]
                dOds[n] = 2.0 * torch.sum(torch.conj(gamma.to(torch.complex128)) * self._apply_S(dpsi)).real
                # co-state one step back: exp(+i dt A_n) in balanced coordinates
                self.h.advance(gamma, svals[n:n + 1], -self.dt)
        dOds = dOds.cpu().numpy()
        return self.W.T @ dOds, dOds


class ObservableFunction:
    """torch.autograd.Function: samples (float64 tensor) -> O(psi_T(samples)).

    Usage:  O = ObservableFunction.apply(samples, adjoint_propagator, psi0, states)
    """

    _impl = None

    @staticmethod
    def _cls():
        if ObservableFunction._impl is None:
            import torch

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, samples, prop, psi0, states):
                    psi_T = prop.forward(psi0, samples.detach().cpu().numpy(), keep=True)
                    # this call's own checkpoints and field values: later forward calls through
                    # the same propagator (several losses, line searches) do not disturb them
                    ctx.prop, ctx.states, ctx.psi_T, ctx.tape = prop, states, psi_T, prop.tape()
                    return torch.tensor(prop.observable(psi_T, states), dtype=torch.float64)

                @staticmethod
                def backward(ctx, grad_out):
                    g, _ = ctx.prop.gradient(ctx.psi_T, ctx.states, tape=ctx.tape)
                    return torch.as_tensor(g, dtype=torch.float64) * grad_out, None, None, None

            ObservableFunction._impl = _F
        return ObservableFunction._impl

    @staticmethod
    def apply(samples, prop, psi0, states):
        return ObservableFunction._cls().apply(samples, prop, psi0, states)
