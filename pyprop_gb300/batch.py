"""Batches of independent hydrogen-like problems advanced together on one GPU.

Each problem is a rank-2 (angular l, radial B-spline) velocity-gauge problem
with its own sizes, pulse, Krylov size and time step.  Its operator is built
directly in the reference storage (one static Diag_BandNH potential, one
time-dependent Simp_BandNH potential), with the same matrix elements the
config-driven TensorPotential generation produces:
  kinetic + centrifugal + Coulomb   examples/tensor/helium_stabilization_sae/potential.cpp:7-33,219-253,
                                    examples/tensor/reducedspherical/potential.cpp:251-282
  velocity-gauge dipole (3 parts)   helium_stabilization_sae/potential.cpp:111-217, config.ini:119-140
The radial band matrices are computed once per problem (not once per angular
point), which is what makes setting up hundreds of problems practical.

All problems share one precision; the batch runs through libgbprop's batch API
(one CUDA graph launch per batch step, the problems as its parallel branches).
"""
from __future__ import annotations

import math

import numpy as np

from . import _native
from .basis import bspline as _bs
from .basis import sphharm as _sph
from .tensorpotential import diagonals_to_bandnh



_ANGULAR = {}


def _angular_dipole(lmax):
    """Dipole selection-rule pairs of l = 0..lmax (m = 0) and the angular factors of the two
    velocity-gauge terms, <l|cos|l'> and <l|d/dtheta-term|l'> by the theta quadrature of
    RepresentPotentialInBasisReducedSphericalHarmonic (basis_reducedspherical.h:11-74); they
    depend on lmax only, so a batch computes them once per distinct lmax."""
    if lmax not in _ANGULAR:
        tools = _sph.ReducedSphericalTools(lmax, 0)
        pairs = _sph.selection_rule_pairs(tools)
        cos_t = np.cos(tools.theta)[:, None]
        ones = np.ones_like(cos_t)
        c_cos = _sph.project_angular(tools, cos_t, pairs, 0)[:, 0]
        c_der = _sph.project_angular(tools, ones, pairs, 1)[:, 0]
        _ANGULAR[lmax] = (pairs, c_cos, c_der)
    return _ANGULAR[lmax]


class HydrogenProblem:
    """One hydrogen-like problem: l = 0..lmax (m = 0), nr B-splines of `order`
    on linear breakpoints over [0, rmax] (zero at both ends), H(t) = H0 + A(t) Hv,
    A(t) = A0 sin^2(pi t / T) (-cos(omega t)) on [0, T), A0 = E0 / omega."""

    def __init__(self, lmax, nr, rmax, order=7, omega=0.057, e0=0.05, cycles=8, m=20, dt=0.01, seed=0,
                 charge=-1.0, setup="host"):
        self.lmax, self.nr, self.rmax, self.order = int(lmax), int(nr), float(rmax), int(order)
        self.omega, self.e0, self.cycles = float(omega), float(e0), float(cycles)
        self.m, self.dt, self.seed, self.charge = int(m), complex(dt), int(seed), float(charge)
        if setup not in ("host", "gpu"):
            raise ValueError("setup must be 'host' or 'gpu'")
        self.setup = setup
        self.amplitude = self.e0 / self.omega
        self.pulse_duration = 2 * math.pi / self.omega * self.cycles
        # zero continuity at both ends: count = nbreak + order - 4 (interior multiplicity 1)
        nbreak = self.nr - self.order + 4
        bps = _bs.linear_breakpoints(0.0, self.rmax, nbreak)
        self.bspline = _bs.BSplineBasis(bps, self.order, _bs.continuity_sequence(nbreak, self.order, "zero"))
        if self.bspline.count != self.nr:
            raise ValueError("B-spline count %d != %d" % (self.bspline.count, self.nr))
        self._build()

    @property
    def nl(self):
        return self.lmax + 1

    @property
    def N(self):
        return self.nl * self.nr

    def _build(self):
        bs = self.bspline
        k = self.order - 1
        g = bs.grid
        n = self.nr
        if self.setup == "gpu":
            # the six radial matrices and the overlap's Cholesky factor in one GPU call
            # (gbprop_bspline_bands; the same quadrature and roundings as the host path below)
            (self.Sdiag, K2, C2, C1, D1, R1), self.Ud = _native.bspline_bands(bs, [
                (_native.RADIAL_CONST, 0, 1.0), (_native.RADIAL_CONST, 2, -0.5), (_native.RADIAL_INV_2R2, 0, 1.0),
                (_native.RADIAL_INV_R, 0, -1.0), (_native.RADIAL_CONST, 1, 1.0), (_native.RADIAL_INV_R, 0, 1.0)],
                cholesky=True)
        else:
            self.Sdiag = bs.band_diagonals(np.ones(len(g)), 0)
            self.Ud = _bs.band_cholesky_upper_diagonals(self.Sdiag, k)
            K2 = bs.band_diagonals(np.full(len(g), -0.5), 2)
            C2 = bs.band_diagonals(1.0 / (2.0 * g * g), 0)
            C1 = bs.band_diagonals(-1.0 / g, 0)
            D1 = bs.band_diagonals(np.ones(len(g)), 1)
            R1 = bs.band_diagonals(1.0 / g, 0)
        K2v, C2v, C1v = diagonals_to_bandnh(K2, k), diagonals_to_bandnh(C2, k), diagonals_to_bandnh(C1, k)
        ls = np.arange(self.nl, dtype=float)
        self.static = (K2v[None, :] + (ls * (ls + 1.0))[:, None] * C2v[None, :] + C1v[None, :]).astype(np.complex128)
        self.pairs, c_cos, c_der = _angular_dipole(self.lmax)
        q = self.charge
        Dv = diagonals_to_bandnh(D1, k)
        Rv = diagonals_to_bandnh(R1, k)
        # charge*i*cos*d/dr  -  charge*i*(1/r)*deriv  -  charge*i*cos/r
        self.dipole = (1j * q * c_cos[:, None] * Dv[None, :] - 1j * q * c_der[:, None] * Rv[None, :]
                       - 1j * q * c_cos[:, None] * Rv[None, :])
        self.kb = k
        self.kd = k
        del n

    def cholesky_band(self):
        """U in the reference's upper band storage: U(i, j) at j*(kd+1) + kd + i - j."""
        n, kd = self.nr, self.kd
        out = np.zeros(n * (kd + 1))
        for d in range(kd + 1):
            i = np.arange(n - d)
            out[(i + d) * (kd + 1) + kd - d] = self.Ud[d, : n - d]
        return out

    def overlap_norm2(self, c):
        """sum_l c_l^H S c_l from the overlap diagonals."""
        kd = self.kd
        n = self.nr
        tot = 0.0
        for d in range(-kd, kd + 1):
            i = np.arange(max(0, -d), min(n, n - d))
            tot += np.sum(np.conj(c[:, i]) * self.Sdiag[kd + d, i] * c[:, i + d]).real
        return tot

    def field(self, t):
        """LaserFunctionVelocity (examples/tensor/helium_stabilization_sae/example.py:220-230)."""
        if 0 <= t < self.pulse_duration:
            return float(self.amplitude * math.sin(t * math.pi / self.pulse_duration) ** 2 * -math.cos(t * self.omega))
        return 0.0

    def initial_state(self):
        """Seeded complex Gaussian coefficients normalised so that psi^H (I x S) psi = 1."""
        rng = np.random.default_rng(self.seed)
        c = rng.standard_normal((self.nl, self.nr)) + 1j * rng.standard_normal((self.nl, self.nr))
        return c / np.sqrt(self.overlap_norm2(c))

    def potentials(self):
        """(storage, pairs, data, time_dependent) in the reference storage."""
        return [(_native.STORAGE_DIAG, None, self.static, False), (_native.STORAGE_SIMP, self.pairs, self.dipole, True)]

    def handle(self, precision=_native.FP64, stream=0):
        h = _native.Handle(self.nl, self.nr, precision, self.m, 0, False, stream)
        h.set_overlap(self.kd, self.cholesky_band())
        for storage, pairs, data, td in self.potentials():
            h.add_potential(storage, pairs, self.kb, data, td)
        h.finalize()
        return h


def random_batch(count=256, seed=20261204, lmax=(8, 64), nr=(200, 1500), rmax=(100.0, 400.0),
                 omega=(0.04, 0.12), e0=(0.02, 0.1), msizes=(16, 24, 32), dt=0.01, order=7, cycles=8, setup="host"):
    """Seeded uneven batch: l_max ~ U{lmax}, Nr ~ U{nr}, r_max ~ U[rmax], omega ~ U[omega],
    E0 ~ U[e0], m in msizes.  setup = "gpu" forms the radial matrices on the GPU."""
    rng = np.random.default_rng(seed)
    probs = []
    for p in range(count):
        probs.append(HydrogenProblem(
            lmax=int(rng.integers(lmax[0], lmax[1] + 1)), nr=int(rng.integers(nr[0], nr[1] + 1)),
            rmax=float(rng.uniform(*rmax)), order=order, omega=float(rng.uniform(*omega)),
            e0=float(rng.uniform(*e0)), cycles=cycles, m=int(rng.choice(msizes)), dt=dt, seed=seed + 1 + p,
            setup=setup))
    return probs


def step_bytes(problem, elem=16):
    """Algorithmic bytes of one Krylov step of a problem: s * N * (m^2 + 7m + 3) (the fused
    step's minimum: the m matvecs' vectors, the Gram-Schmidt passes over the basis, the final
    combination)."""
    return elem * problem.N * (problem.m * problem.m + 7 * problem.m + 3)


def shard(problems, world, elem=16):
    """Split one batch over `world` GPUs with no communication during propagation: greedy
    bin-packing by the per-step work (largest first onto the least-loaded rank, ties to the lower
    rank).  Returns one sorted list of problem indices per rank; every problem is on exactly one
    rank.  Deterministic, so every rank computes the same plan without exchanging it."""
    order = sorted(range(len(problems)), key=lambda i: (-step_bytes(problems[i], elem), i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += step_bytes(problems[i], elem)
    return [sorted(x) for x in out]


def gather_states(states, indices, world, count):
    """All ranks' final states back in batch order on rank 0 (host numpy arrays; a list of
    `count` arrays on rank 0, None elsewhere).  `indices` are this rank's problems (shard())."""
    if world == 1:
        out = [None] * count
        for i, x in zip(indices, states):
            out[i] = x
        return out
    import torch.distributed as dist
    mine = list(zip(indices, states))
    allp = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(mine, allp, dst=0)
    if dist.get_rank() != 0:
        return None
    out = [None] * count
    for part in allp:
        for i, x in part:
            out[i] = x
    return out


class BatchPropagator:
    """Advances a list of HydrogenProblem together: one batch step = one
    PamPropagator step of every problem (each with its own field and dt)."""

    def __init__(self, problems, precision=_native.FP64, autotune=True, device="cuda"):
        import torch
        self.problems = list(problems)
        self.precision = precision
        stream = torch.cuda.current_stream().cuda_stream
        self.handles = [p.handle(precision, stream) for p in self.problems]
        cdt = torch.complex128 if precision == _native.FP64 else torch.complex64
        self.psi = [torch.as_tensor(p.initial_state()).to(device, cdt) for p in self.problems]
        self.batch = _native.Batch(self.handles, autotune=autotune, stream=stream)
        self.time = [0.0] * len(self.problems)

    def advance(self, nsteps):
        P = len(self.problems)
        scal = np.zeros((P, nsteps))
        for p, prob in enumerate(self.problems):
            t = self.time[p]
            for n in range(nsteps):
                scal[p, n] = prob.field(t)
                t = t + prob.dt.real
            self.time[p] = t
        self.batch.advance(self.psi, scal, [p.dt for p in self.problems])

    def synchronize(self):
        """Wait for the batch; raises GbpropError for a device-side failure of any problem."""
        self.batch.synchronize()

    def scalings(self, p, nsteps, t0=0.0):
        prob = self.problems[p]
        out, t = [], t0
        for _ in range(nsteps):
            out.append(prob.field(t))
            t = t + prob.dt.real
        return np.array(out)
