"""Grid potentials named by `classname` in TensorPotential config sections.

Each entry evaluates V(angular coordinate, r) on a tensor grid.  The angular
coordinate is l for a Diagonal angular geometry (the basis representation,
GeometryInfo "Diag" uses the basis values) and theta for the dipole
selection rule (grid representation).  Definitions follow the reference's
example potentials:
  KineticEnergyPotential, KineticEnergyPotential2, AngularKineticEnergyPotential,
  DipoleLaserPotentialLength, DipoleLaserPotentialVelocity{,RadialDerivative,AngularDerivative},
  SingleActiveElectronPotential
      examples/tensor/helium_stabilization_sae/potential.cpp:6-330
  RadialCoulombPotential
      examples/tensor/reducedspherical/potential.cpp:251-282
A classname that is not listed is looked up in the project namespace: a
callable `f(section, ang, r)` returning an array of the grid shape.
"""
from __future__ import annotations

import numpy as np


def _kinetic(sec, ang, r):
    return np.full(np.broadcast(ang, r).shape, -1.0 / (2.0 * sec.mass))


def _kinetic2(sec, ang, r):
    return -1.0 / (sec.mass * np.sqrt(r * r + sec.soft * sec.soft)) + 0.0 * ang


def _angular_kinetic(sec, l, r):
    return l * (l + 1.0) / (2.0 * sec.mass * r * r)


def _coulomb(sec, ang, r):
    return -1.0 / r + 0.0 * ang


def _dipole_length(sec, theta, r):
    return -sec.charge * r * np.cos(theta)


def _dipole_velocity_radial_derivative(sec, theta, r):
    return sec.charge * 1j * np.cos(theta) + 0.0 * r


def _dipole_velocity_angular_derivative(sec, theta, r):
    return -sec.charge * 1j / r + 0.0 * theta


def _dipole_velocity(sec, theta, r):
    return -sec.charge * 1j * np.cos(theta) / r


def _sae(sec, ang, r):
    r = np.abs(r)
    return (-(sec.z + sec.a1 * np.exp(-sec.a2 * r) + sec.a3 * r * np.exp(-sec.a4 * r)
              + sec.a5 * np.exp(-sec.a6 * r)) / np.sqrt(r * r + sec.soft * sec.soft)) + 0.0 * ang


POTENTIALS = {
    "KineticEnergyPotential": _kinetic,
    "KineticEnergyPotential2": _kinetic2,
    "AngularKineticEnergyPotential": _angular_kinetic,
    "RadialCoulombPotential": _coulomb,
    "DipoleLaserPotentialLength": _dipole_length,
    "DipoleLaserPotentialVelocityRadialDerivative": _dipole_velocity_radial_derivative,
    "DipoleLaserPotentialVelocityAngularDerivative": _dipole_velocity_angular_derivative,
    "DipoleLaserPotentialVelocity": _dipole_velocity,
    "SingleActiveElectronPotential": _sae,
}


def evaluate(section, ang, r):
    """Evaluate the potential of `section` on the tensor grid ang[:, None] x r[None, :]."""
    name = section.classname
    fn = POTENTIALS.get(name)
    if fn is None:
        from .config import _project_namespace
        fn = _project_namespace().get(name)
        if fn is None or not callable(fn):
            raise KeyError("unknown potential classname %r" % (name,))
    A = np.asarray(ang, dtype=float)[:, None]
    R = np.asarray(r, dtype=float)[None, :]
    v = np.asarray(fn(section, A, R))
    return np.broadcast_to(v, (A.shape[0], R.shape[1])).copy()


# ---------------------------------------------------------------------------
# time functions (the reference defines these in its example scripts and
# names them in `time_function = ...`; examples/tensor/helium_stabilization_sae/example.py:220-241)
# ---------------------------------------------------------------------------
def LaserFunctionVelocity(conf, t):
    """A(t) = A0 sin^2(pi t / T) * (-cos(omega t + phase)) on [0, T), zero outside."""
    phase = getattr(conf, "phase", 0.0)
    if 0 <= t < conf.pulse_duration:
        cur = conf.amplitude
        cur *= np.sin(t * np.pi / conf.pulse_duration) ** 2
        cur *= -np.cos(t * conf.frequency + phase)
    else:
        cur = 0.0
    return float(cur)


def LaserFunctionSimpleLength(conf, t):
    """E(t) = E0 sin^2(pi t / T) cos(omega t) on [0, T), zero outside."""
    if 0 <= t < conf.pulse_duration:
        cur = conf.amplitude
        cur *= np.sin(t * np.pi / conf.pulse_duration) ** 2
        cur *= np.cos(t * conf.frequency)
    else:
        cur = 0.0
    return float(cur)


def PiecewiseLinearField(conf, t):
    """Piecewise-linear interpolation of `field_samples` on a uniform grid over
    [0, pulse_duration]; zero outside.  The control used by the adjoint."""
    samples = np.asarray(conf.field_samples, dtype=float)
    T = conf.pulse_duration
    if not (0 <= t <= T) or len(samples) == 0:
        return 0.0
    if len(samples) == 1:
        return float(samples[0])
    x = t / T * (len(samples) - 1)
    k = min(int(np.floor(x)), len(samples) - 2)
    w = x - k
    return float((1.0 - w) * samples[k] + w * samples[k + 1])
