"""Names visible to evaluated config values (pyprop/__init__.py:17-27 puts
numpy and the pyprop classes in the namespace config expressions see)."""
from __future__ import annotations

import types

import numpy as _np


class PotentialType:
    """pyprop/Enum.py potential types; only TensorPotential sections are used on this path."""
    Static = "Static"
    Dynamic = "Dynamic"
    RankOne = "RankOne"
    FiniteDifference = "FiniteDifference"
    Matrix = "Matrix"


def _core_namespace():
    from .representation import (BSplineRepresentation, CombinedRepresentation,
                                 ReducedSphericalHarmonicRepresentation)

    class CombinedRepresentation_2(CombinedRepresentation):
        def __init__(self, rank=2):
            CombinedRepresentation.__init__(self, rank)

    core = types.SimpleNamespace(
        CombinedRepresentation_2=CombinedRepresentation_2,
        ReducedSphericalHarmonicRepresentation=ReducedSphericalHarmonicRepresentation,
        BSplineRepresentation=BSplineRepresentation,
    )
    return core


_CACHE = {}


def eval_namespace():
    if "ns" in _CACHE:
        return _CACHE["ns"]
    ns = {}
    for k in dir(_np):
        if not k.startswith("_"):
            ns[k] = getattr(_np, k)
    from . import potentials, problem, propagator, initial
    ns["core"] = _core_namespace()
    ns["PotentialType"] = PotentialType
    ns["InitialConditionType"] = problem.InitialConditionType
    ns["WavefunctionFileFormat"] = problem.WavefunctionFileFormat
    ns["PamPropagator"] = propagator.PamPropagator
    ns["ExpokitPropagator"] = propagator.ExpokitPropagator
    ns["BasisPropagator"] = propagator.BasisPropagator
    ns["LaserFunctionVelocity"] = potentials.LaserFunctionVelocity
    ns["LaserFunctionSimpleLength"] = potentials.LaserFunctionSimpleLength
    ns["PiecewiseLinearField"] = potentials.PiecewiseLinearField
    ns["GaussianRandomState"] = initial.GaussianRandomState
    ns["InitBSpline"] = None
    _CACHE["ns"] = ns
    return ns
