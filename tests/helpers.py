"""Shared builders for the parity tests."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CONFIG_TEMPLATE = """
[Representation]
rank = 2
type = core.CombinedRepresentation_2
representation0 = "AngularRepresentation"
representation1 = "RadialRepresentation"

[AngularRepresentation]
type = core.ReducedSphericalHarmonicRepresentation
maxl = {maxl}
m = 0

[RadialRepresentation]
type = core.BSplineRepresentation
xmin = 0.0
xmax = {xmax}
xsize = {xsize}
bpstype = '{bpstype}'
xpartition = {xpartition}
gamma = {gamma}
continuity = 'zero'
order = {order}
quad_order_additional = 0
projection_algorithm = 0

[InitialCondition]
type = InitialConditionType.Custom
function = GaussianRandomState
seed = {seed}

[PulseParameters]
frequency = {omega}
cycles = {cycles}
pulse_duration = 2 * pi / %(frequency)s * %(cycles)s
amplitude = {e0} / %(frequency)s

[Propagation]
base = "PulseParameters"
potential_evaluation = []
grid_potential_list = {potentials}
propagator = PamPropagator
base_propagator = BasisPropagator
timestep = {dt}
duration = {duration}
renormalization = {renorm}
krylov_basis_size = {m}
krylov_double_orthogonalization = {dorth}
krylov_precision = "{precision}"
silent = True

[RadialKineticEnergy]
classname = "KineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
differentiation0 = 0
differentiation1 = 2
mass = 1

[AngularKineticEnergy]
classname = "AngularKineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
mass = 1
angular_rank = 0
radial_rank = 1

[CoulombPotential]
classname = "RadialCoulombPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
angular_rank = 0
radial_rank = 1

[LaserPotentialVelocityBase]
base = "PulseParameters"
geometry0 = "dipoleselectionrule"
geometry1 = "banded-nonhermitian"
angular_rank = 0
radial_rank = 1
time_function = LaserFunctionVelocity
charge = -1.0

[LaserPotentialVelocity1]
base = "LaserPotentialVelocityBase"
classname = "DipoleLaserPotentialVelocityRadialDerivative"
differentiation1 = 1

[LaserPotentialVelocity2]
base = "LaserPotentialVelocityBase"
classname = "DipoleLaserPotentialVelocityAngularDerivative"
differentiation0 = 1

[LaserPotentialVelocity3]
base = "LaserPotentialVelocityBase"
classname = "DipoleLaserPotentialVelocity"
"""

ALL_POTENTIALS = ["RadialKineticEnergy", "AngularKineticEnergy", "CoulombPotential",
                  "LaserPotentialVelocity1", "LaserPotentialVelocity2", "LaserPotentialVelocity3"]


def config_text(maxl=3, xmax=20.0, xsize=30, order=7, m=8, dt=0.01, duration=0.1, seed=7, omega=0.057,
                cycles=8, e0=0.05, precision="fp64", dorth=False, renorm=False, potentials=None,
                bpstype="linear", xpartition=5.0, gamma=2.0):
    return CONFIG_TEMPLATE.format(maxl=maxl, xmax=xmax, xsize=xsize, order=order, m=m, dt=dt, duration=duration,
                                  seed=seed, omega=omega, cycles=cycles, e0=e0, precision=precision, dorth=dorth,
                                  renorm=renorm, potentials=repr(potentials or ALL_POTENTIALS), bpstype=bpstype,
                                  xpartition=xpartition, gamma=gamma)


def make_problem(device="cuda", setup=True, **kw):
    import pyprop_gb300 as pp
    conf = pp.LoadString(config_text(**kw))
    prob = pp.Problem(conf, device=device)
    if setup:
        prob.SetupStep()
    else:
        prob.SetupWavefunction()
    return prob


def step_times(prob, n):
    times = []
    t = prob.PropagatedTime
    for _ in range(n):
        times.append(t)
        t = prob._next_time(t)
    return times


def scalings_for(prob, n):
    bp = prob.Propagator.BasePropagator
    return np.array([bp._scaling(t) for t in step_times(prob, n)])


def rel(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
