"""Propagators: PropagatorBase, BasisPropagator and PamPropagator.

Same classes, methods, config keys and call order as the reference:
  PropagatorBase   pyprop/propagator/Propagator.py:5-81
  BasisPropagator  pyprop/tensorpotential/BasisPropagator.py:1-165
  PamPropagator    pyprop/propagator/PamPropagator.py:2-83
  PampWrapper keys core/krylov/pamp/pampwrapper.cpp:50-70
The Krylov step (pAMP Arnoldi + Pade exponential) and the balanced-overlap
TensorPotential matvec run on the GPU through libgbprop; nothing here falls
back to a CPU implementation.
"""
from __future__ import annotations

import numpy as np

from . import _native
from .tensorpotential import generate_potentials

_STORAGE = {"Diag": _native.STORAGE_DIAG, "Ident": _native.STORAGE_IDENT, "Simp": _native.STORAGE_SIMP}
_PRECISION = {"fp64": _native.FP64, "double": _native.FP64, "fp32-mixed": _native.FP32_MIXED,
              "fp32_mixed": _native.FP32_MIXED, "mixed": _native.FP32_MIXED}


def precision_of(name):
    key = str(name).lower()
    if key not in _PRECISION:
        raise ValueError("unknown krylov_precision %r (fp64 | fp32-mixed)" % (name,))
    return _PRECISION[key]


def _require_device(psi):
    if psi.data.device.type != "cuda":
        raise RuntimeError("the propagation path runs on the GPU only: wavefunction is on %s" % psi.data.device)


MAX_TIME_FUNCTIONS = 4


def time_function_numbers(potentials):
    """The time-function number of every consolidated potential: 0 for static ones, and
    1, 2, ... for the time-dependent ones in list order.  Each consolidated potential keeps its
    own time function, evaluated with its own config section (TensorPotential.py:98-100, looped
    by Propagator.py:61-66); consolidation has already merged potentials sharing one."""
    nums, k = [], 0
    for p in potentials:
        if p.IsTimeDependent:
            k += 1
            nums.append(k)
        else:
            nums.append(0)
    if k > MAX_TIME_FUNCTIONS:
        raise NotImplementedError("%d time-dependent TensorPotentials after consolidation; at most %d"
                                  % (k, MAX_TIME_FUNCTIONS))
    return nums


def build_handle(psi, potentials, precision=_native.FP64, krylov_basis_size=1, exponentiation_method=0,
                 double_orthogonalization=False):
    """Create and finalize a libgbprop handle for the wavefunction's
    representation and a consolidated TensorPotential list."""
    import torch
    repr_ = psi.GetRepresentation()
    nl, nr = repr_.GetFullShape()
    tf = time_function_numbers(potentials)
    stream = torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else 0
    h = _native.Handle(nl, nr, precision, krylov_basis_size, exponentiation_method, double_orthogonalization, stream)
    h.set_overlap(repr_.radial.kd, repr_.radial.cholesky_band())
    for p, k in zip(potentials, tf):
        s0, s1 = p.GetStorageIds()
        if s1 != "BandNH":
            raise NotImplementedError("radial storage %s" % s1)
        pairs = p.GeometryList[0].GetBasisPairs() if s0 == "Simp" else None
        h.add_potential(_STORAGE[s0], pairs, p.GeometryList[1].band_count, p.PotentialData, k)
    h.finalize()
    return h


class PropagatorBase:
    def __init__(self, psi):
        self.psi = psi
        self.RenormalizeActive = False
        self.PotentialList = []

    def ApplyConfig(self, config):
        names = getattr(config.Propagation, "potential_evaluation", [])
        if names:
            raise NotImplementedError("grid potentials (potential_evaluation) are outside the propagation path "
                                      "provided here; use TensorPotentials in grid_potential_list")
        self.PotentialList = []

    def ApplyConfigSection(self, sec):
        self.RenormalizeActive = bool(getattr(sec, "renormalization", False))

    def SetupStep(self, dt):
        pass

    def RestartPropagation(self, timestep, startTime, propagationTime):
        pass

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        raise NotImplementedError("MultiplyHamiltonian should be implemented by %s" % self.__class__)


class BasisPropagator(PropagatorBase):
    """Applies TensorPotentials in the basis (BasisPropagator.py:1-165)."""

    def __init__(self, psi):
        PropagatorBase.__init__(self, psi)
        self.PotentialList = []
        self._handle = None

    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        names = list(getattr(config.Propagation, "grid_potential_list", []))
        self.PotentialList = generate_potentials(self.psi, config, names)

    def ApplyConfigSection(self, sec):
        PropagatorBase.ApplyConfigSection(self, sec)

    def SetupStep(self, dt):
        pass

    def AttachHandle(self, handle):
        self._handle = handle

    def Handle(self):
        if self._handle is None:
            prec = _native.FP64 if self.psi.data.dtype.itemsize == 16 else _native.FP32_MIXED
            self._handle = build_handle(self.psi, self.PotentialList, prec, 1)
        return self._handle

    def _scalings_at(self, t):
        """The time functions at t, in time-function-number order (time_function_numbers);
        [1.0] when no potential is time dependent."""
        vals = [p.GetScaling(t) for p in self.PotentialList if p.IsTimeDependent]
        return np.array(vals or [1.0], dtype=np.float64)

    def _scaling(self, t):
        """The time function at t, for operators with at most one (the reference's single-pulse
        configurations); see _scalings_at for several."""
        v = self._scalings_at(t)
        if len(v) > 1:
            raise ValueError("%d time functions: use _scalings_at" % len(v))
        return float(v[0])

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        """dest = S^-1 H(t) src (BasisPropagator.py:116-124; SolveOverlap = U^-1 U^-T)."""
        _require_device(srcPsi)
        h = self.Handle()
        h.matvec(srcPsi.data, destPsi.data, self._scalings_at(t), balanced=False)
        h.solve_sqrt_overlap(True, destPsi.data)
        h.solve_sqrt_overlap(False, destPsi.data)

    def MultiplyHamiltonianNoOverlap(self, srcPsi, destPsi, t, dt):
        _require_device(srcPsi)
        self.Handle().matvec(srcPsi.data, destPsi.data, self._scalings_at(t), balanced=False)

    def MultiplyHamiltonianBalancedOverlap(self, srcPsi, destPsi, t, dt):
        _require_device(srcPsi)
        self.Handle().matvec(srcPsi.data, destPsi.data, self._scalings_at(t), balanced=True)

    def AdvanceStep(self, t, dt):
        raise NotImplementedError("BasisPropagator does not support AdvanceStep. Use it as a base for explicit propagators")


class _PampCounters:
    """The counters krylov_PampWrapper exposes (pampwrapper.h:169-237)."""

    def __init__(self, owner):
        self._owner = owner

    def _stats(self):
        return self._owner._handle.stats()

    def GetOperatorCount(self):
        return int(self._stats().operator_count)

    def GetOrthogonalizationCount(self):
        return int(self._stats().orthogonalization_count)

    def GetPropagationErrorEstimate(self):
        return float(self._stats().error_estimate)

    def GetHessenbergMatrix(self):
        return self._owner._handle.hessenberg()

    def ResetStatistics(self):
        self._owner._handle.reset_stats()

    def PrintStatistics(self):
        s = self._stats()
        print("    OpCount      = %d" % s.operator_count)
        print("    InnerProduct = %d" % s.inner_product_count)
        print("    ReOrthoCOunt = %d" % s.orthogonalization_count)


class PamPropagator(PropagatorBase):
    """pAMP Krylov propagator around the balanced-overlap TensorPotential matvec."""

    RenormalizesOnDevice = True     # renormalization = True is applied inside every device step

    def __init__(self, psi):
        PropagatorBase.__init__(self, psi)
        self.Rank = psi.GetRank()
        self.BasisSize = 20
        self.ExponentiationMethod = 0
        self.DoubleOrthogonalization = False
        self.Precision = _native.FP64
        self.Autotune = True
        self.BandVariant = None
        self._handle = None
        self.PampWrapper = _PampCounters(self)

    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        propagatorType = config.Propagation.base_propagator
        self.BasePropagator = propagatorType(self.psi)
        config.Apply(self.BasePropagator)

    def ApplyConfigSection(self, sec):
        PropagatorBase.ApplyConfigSection(self, sec)
        sec.Apply(self.BasePropagator)
        self.BasisSize = int(sec.krylov_basis_size)
        if hasattr(sec, "krylov_exponentiation_method"):
            self.ExponentiationMethod = int(sec.krylov_exponentiation_method)
        if hasattr(sec, "krylov_double_orthogonalization"):
            self.DoubleOrthogonalization = bool(sec.krylov_double_orthogonalization)
        if hasattr(sec, "krylov_precision"):
            self.Precision = precision_of(sec.krylov_precision)
        if hasattr(sec, "krylov_autotune"):
            self.Autotune = bool(sec.krylov_autotune)

    def SetupStep(self, dt):
        self.BasePropagator.SetupStep(dt)
        _require_device(self.psi)
        self._handle = build_handle(self.psi, self.BasePropagator.PotentialList, self.Precision, self.BasisSize,
                                    self.ExponentiationMethod, self.DoubleOrthogonalization)
        # renormalization = True: every step ends with psi.Normalize() on the device
        self._handle.set_renormalization(self.RenormalizeActive)
        if self.Autotune:
            # pick the band kernel's tile shape for this operator
            self.BandVariant = self._handle.autotune()
        self.BasePropagator.AttachHandle(self._handle)
        self.psi.AttachHandle(self._handle)
        self.TempPsi = self.psi.CopyDeep()

    def _scalings(self, times):
        """(len(times), K): the K time functions at the start of every step."""
        return np.array([self.BasePropagator._scalings_at(t) for t in times], dtype=np.float64)

    def AdvanceStep(self, t, dt):
        self.AdvanceSteps([t], dt)

    def AdvanceSteps(self, times, dt):
        """len(times) consecutive AdvanceStep calls, step n at t = times[n], in one device submission."""
        if self._handle is None:
            raise RuntimeError("SetupStep must be called before AdvanceStep")
        self._handle.advance(self.psi.data, self._scalings(times), dt)

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        self.BasePropagator.MultiplyHamiltonian(srcPsi, destPsi, t, dt)

    def Handle(self):
        return self._handle


class ExpokitPropagator(PropagatorBase):
    """Expokit Krylov propagator (pyprop/propagator/KrylovPropagator.py:2-58): the same
    balanced-overlap matvec inside zgexpv's adaptive sub-stepping with local error control
    (core/krylov/expokit/expokitpropagator.cpp:18-103).  Keys: krylov_basis_size,
    krylov_tolerance, krylov_norm (an estimate of the operator's norm, used for the first
    sub-step size)."""

    RenormalizesOnDevice = True

    def __init__(self, psi):
        PropagatorBase.__init__(self, psi)
        self.Rank = psi.GetRank()
        self.BasisSize = 20
        self.Tolerance = 0.0
        self.MatrixNorm = 1.0
        self.Precision = _native.FP64
        self.Autotune = True
        self._handle = None
        self.Statistics = None

    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        propagatorType = config.Propagation.base_propagator
        self.BasePropagator = propagatorType(self.psi)
        config.Apply(self.BasePropagator)

    def ApplyConfigSection(self, sec):
        PropagatorBase.ApplyConfigSection(self, sec)
        sec.Apply(self.BasePropagator)
        self.BasisSize = int(sec.krylov_basis_size)
        self.Tolerance = float(sec.krylov_tolerance)
        self.MatrixNorm = float(sec.krylov_norm)
        if hasattr(sec, "krylov_precision"):
            self.Precision = precision_of(sec.krylov_precision)
        if hasattr(sec, "krylov_autotune"):
            self.Autotune = bool(sec.krylov_autotune)

    def SetupStep(self, dt):
        self.BasePropagator.SetupStep(dt)
        _require_device(self.psi)
        # m + 1 basis vectors: zgexpv's extra operator application A v_{m+1}
        self._handle = build_handle(self.psi, self.BasePropagator.PotentialList, self.Precision,
                                    self.BasisSize + 1, 0, True)
        self._handle.set_renormalization(self.RenormalizeActive)
        if self.Autotune:
            self._handle.autotune()
        self.BasePropagator.AttachHandle(self._handle)
        self.psi.AttachHandle(self._handle)
        self.TempPsi = self.psi.CopyDeep()

    def AdvanceStep(self, t, dt):
        self.AdvanceSteps([t], dt)

    def AdvanceSteps(self, times, dt):
        if self._handle is None:
            raise RuntimeError("SetupStep must be called before AdvanceStep")
        scal = np.array([self.BasePropagator._scalings_at(t) for t in times], dtype=np.float64)
        self.Statistics = self._handle.expokit_advance(self.psi.data, scal, dt, self.Tolerance, self.MatrixNorm)

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        self.BasePropagator.MultiplyHamiltonian(srcPsi, destPsi, t, dt)

    def Handle(self):
        return self._handle
