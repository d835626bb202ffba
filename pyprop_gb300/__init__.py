"""pyprop_gb300: pyprop's pAMP x TensorPotential propagation step on GB300.

The Python surface mirrors pyprop's: Load, Problem, LoadPropagator,
PamPropagator, BasisPropagator, TensorPotential, with the same INI keys.  The
step itself runs in libgbprop (CUDA, sm_103a) behind a C ABI (include/gbprop.h).
"""
from .config import Config, Load, LoadString, Section
from .initial import GaussianRandomState
from .potentials import LaserFunctionSimpleLength, LaserFunctionVelocity, PiecewiseLinearField
from .problem import InitialConditionType, LoadPropagator, Problem, WavefunctionFileFormat
from .propagator import BasisPropagator, ExpokitPropagator, PamPropagator, PropagatorBase
from .representation import (BSplineRepresentation, CombinedRepresentation, ReducedSphericalHarmonicRepresentation,
                             Wavefunction)
from .tensorpotential import TensorPotential
from .namespace import PotentialType

__all__ = [
    "Config", "Load", "LoadString", "Section", "Problem", "LoadPropagator", "PamPropagator", "ExpokitPropagator", "BasisPropagator",
    "PropagatorBase", "TensorPotential", "Wavefunction", "CombinedRepresentation", "BSplineRepresentation",
    "ReducedSphericalHarmonicRepresentation", "InitialConditionType", "WavefunctionFileFormat", "PotentialType", "LaserFunctionVelocity",
    "LaserFunctionSimpleLength", "PiecewiseLinearField", "GaussianRandomState",
]
