"""Problem: the user-facing driver (pyprop/Problem.py:55-476, CreateInstance.py:2-151).

    conf = pyprop_gb300.Load("config.ini")
    prop = pyprop_gb300.Problem(conf)        # or pyprop_gb300.LoadPropagator("config.ini")
    prop.SetupStep()
    for t in prop.Advance(10):
        ...

Advance() submits the steps between two yields as one device call (the field
values of those steps are evaluated on the host first, at the times the
per-step loop would use); renormalization, when active, happens inside it.
"""
from __future__ import annotations

import numpy as np

from .config import Load
from .representation import (BSplineRepresentation, CombinedRepresentation, ReducedSphericalHarmonicRepresentation,
                             Wavefunction)


class InitialConditionType:
    Function = "Function"
    File = "File"
    Class = "Class"
    Custom = "Custom"


class WavefunctionFileFormat:
    """File formats of InitialConditionType.File (Enum.py:21-24)."""
    Ascii = 1
    Binary = 2
    HDF = 3


def CreateRepresentation(config):
    """CreateRepresentation + CreateSubRepresentations (CreateInstance.py:42-87)."""
    rsec = config.Representation
    rank = int(rsec.rank)
    combined = rsec.type(rank) if isinstance(rsec.type, type) and issubclass(rsec.type, CombinedRepresentation) \
        else CombinedRepresentation(rank)
    for i in range(rank):
        sec = config.GetSection(rsec.Get("representation%i" % i))
        sub = sec.type()
        sec.Apply(sub)
        combined.SetRepresentation(i, sub)
    if not isinstance(combined.angular, ReducedSphericalHarmonicRepresentation) or \
            not isinstance(combined.radial, BSplineRepresentation):
        raise NotImplementedError("representation must be (ReducedSphericalHarmonic, BSpline)")
    return combined


def CreateWavefunction(config, device=None):
    """CreateWavefunction (Problem.py:5-29); complex64 storage for the mixed path."""
    repr_ = CreateRepresentation(config)
    prec = str(getattr(config.Propagation, "krylov_precision", "fp64")).lower()
    dtype = "complex64" if prec in ("fp32-mixed", "fp32_mixed", "mixed") else "complex128"
    return Wavefunction(repr_, dtype=dtype, device=device)


def CreatePropagator(config, psi):
    """CreatePropagator (CreateInstance.py:107-118)."""
    if not hasattr(config.Propagation, "propagator"):
        print("WARNING: No propagator specified in config file.")
        return None
    propagator = config.Propagation.propagator(psi)
    config.Apply(propagator)
    config.Propagation.Apply(propagator)
    return propagator


class Problem:
    def __init__(self, config, device=None):
        self.TempPsi = None
        self.Config = config
        self.Silent = bool(getattr(config.Propagation, "silent", False))
        self.psi = CreateWavefunction(config, device=device)
        self.Propagator = CreatePropagator(config, self.psi)
        config.Propagation.Apply(self)

    # Problem.ApplyConfigSection (Problem.py:306-314)
    def ApplyConfigSection(self, sec):
        self.TimeStep = complex(sec.timestep)
        self.Duration = sec.duration
        self.PropagatedTime = 0
        self.StartTime = 0
        if hasattr(sec, "start_time"):
            self.StartTime = sec["start_time"]
            self.PropagatedTime = self.StartTime

    def GetGrid(self):
        repr_ = self.psi.GetRepresentation()
        return [np.asarray(repr_.angular.lvalues(), dtype=float), repr_.radial.bspline.grid]

    def SetupStep(self, skipWavefunctionSetup=False):
        if self.Propagator is not None:
            self.Propagator.SetupStep(self.TimeStep)
        if not skipWavefunctionSetup:
            self.SetupWavefunction()

    def RestartPropagation(self, timestep, startTime, propagationTime):
        self.TimeStep = timestep
        self.PropagatedTime = startTime
        self.StartTime = startTime
        self.Duration = propagationTime
        if self.Propagator is not None:
            self.Propagator.RestartPropagation(timestep, startTime, propagationTime)

    def _next_time(self, t):
        # Problem.py:170-173
        if abs(self.TimeStep.real) < 1e-10:
            return t + abs(self.TimeStep)
        return t + self.TimeStep.real

    def AdvanceStep(self):
        """Problem.AdvanceStep (Problem.py:158-173).  With renormalization on, the Krylov
        propagators normalise psi inside the device step (the same psi.Normalize())."""
        self.Propagator.AdvanceStep(self.PropagatedTime, self.TimeStep)
        if self.Propagator.RenormalizeActive and not getattr(self.Propagator, "RenormalizesOnDevice", False):
            self.psi.Normalize()
        self.PropagatedTime = self._next_time(self.PropagatedTime)

    def AdvanceSteps(self, n):
        """n consecutive AdvanceStep calls submitted as one device call."""
        if n <= 0:
            return
        if not hasattr(self.Propagator, "AdvanceSteps") or (
                self.Propagator.RenormalizeActive and not getattr(self.Propagator, "RenormalizesOnDevice", False)):
            for _ in range(n):
                self.AdvanceStep()
            return
        times = []
        t = self.PropagatedTime
        for _ in range(n):
            times.append(t)
            t = self._next_time(t)
        self.Propagator.AdvanceSteps(times, self.TimeStep)
        self.PropagatedTime = t

    def Advance(self, yieldCount, duration=None, yieldEnd=False):
        """Problem.Advance generator (Problem.py:182-240)."""
        if duration is None:
            duration = self.Duration
        if yieldCount.__class__ is bool:
            yieldStep = 1
        else:
            yieldStep = max(1, int((duration / abs(self.TimeStep)) / yieldCount))
        if self.TimeStep.real == 0:
            stop = lambda t: (self.StartTime + self.Duration - t) > 0.5 * abs(self.TimeStep)
        else:
            endTime = self.StartTime + np.sign(self.TimeStep.real) * self.Duration
            stop = lambda t: abs(t - endTime) > 0.5 * abs(self.TimeStep)
        prevYield = np.nan
        index = 0
        while stop(self.PropagatedTime):
            # number of steps until the next yield or the end, by the same clock
            n = 0
            t = self.PropagatedTime
            while stop(t) and (n == 0 or (index + n) % yieldStep != 0):
                t = self._next_time(t)
                n += 1
            self.AdvanceSteps(n)
            index += n
            if index % yieldStep == 0:
                yield self.PropagatedTime
                prevYield = self.PropagatedTime
        if yieldEnd and prevYield != self.PropagatedTime:
            yield self.PropagatedTime

    def MultiplyHamiltonian(self, srcPsi, dstPsi):
        self.Propagator.MultiplyHamiltonian(srcPsi, dstPsi, self.PropagatedTime, self.TimeStep)

    def GetTempPsi(self):
        if self.TempPsi is None:
            self.TempPsi = self.psi.CopyDeep()
        return self.TempPsi

    def GetEnergyExpectationValue(self):
        """Problem.GetEnergyExpectationValue (Problem.py:254-276)."""
        self.psi.Normalize()
        tmp = self.GetTempPsi()
        tmp.Clear()
        self.MultiplyHamiltonian(self.psi, tmp)
        energy = self.psi.InnerProduct(tmp)
        return energy.real

    def GetEnergy(self):
        return self.GetEnergyExpectationValue()

    # initial condition (Problem.py:317-421)
    def SetupWavefunction(self):
        ic = getattr(self.Config, "InitialCondition", None)
        t = getattr(ic, "type", None) if ic is not None else None
        if t is None:
            return
        if t == InitialConditionType.Function:
            self.SetupWavefunctionFunction(self.Config)
        elif t == InitialConditionType.Custom:
            ic.function(self.psi, ic)
        elif t == InitialConditionType.Class:
            obj = ic.classname()
            ic.Apply(obj)
            obj.SetupWavefunction(self.psi)
        elif t == InitialConditionType.File:
            self.SetupWavefunctionFile(self.Config)
        else:
            raise ValueError("Invalid InitialConditionType: %r" % (t,))

    # wavefunction files (Problem.py:397-474): the same grid must be used for saving and loading
    def SetupWavefunctionFile(self, config):
        fmt = config.InitialCondition.format
        filename = config.InitialCondition.filename
        if fmt == WavefunctionFileFormat.Ascii:
            self.LoadWavefunctionAscii(filename)
        elif fmt == WavefunctionFileFormat.Binary:
            self.LoadWavefunctionPickle(filename)
        elif fmt == WavefunctionFileFormat.HDF:
            self.LoadWavefunctionHDF(filename, str(config.InitialCondition.dataset))
        else:
            raise ValueError("Invalid file format: %r" % (fmt,))

    def LoadWavefunctionData(self, newdata):
        newdata = np.asarray(newdata)
        shape = tuple(self.psi.GetData().shape)
        if newdata.shape != shape:
            raise ValueError("Invalid shape on loaded wavefunction, got %s expected %s" % (newdata.shape, shape))
        self.psi.SetData(newdata)

    def SaveWavefunctionPickle(self, filename):
        """The data array pickled with protocol 2 (serialization/Pickle.py:4-13)."""
        import pickle
        with open(filename, "wb") as f:
            pickle.dump(np.ascontiguousarray(self.psi.GetDataNumpy()), f, 2)

    def LoadWavefunctionPickle(self, filename):
        """serialization/Pickle.py:15-27; latin-1 decoding also reads arrays pickled by Python 2."""
        import pickle
        with open(filename, "rb") as f:
            arr = pickle.load(f, encoding="latin1")
        self.LoadWavefunctionData(arr)

    def SaveWavefunctionAscii(self, filename):
        """Two columns, real and imaginary part (Problem.py:457-460), of the C-ordered data (the
        reference writes rank-1 data only)."""
        d = self.psi.GetDataNumpy().ravel()
        np.savetxt(filename, np.column_stack((d.real, d.imag)), delimiter=" ")

    def LoadWavefunctionAscii(self, filename):
        r, c = np.loadtxt(filename, unpack=True, ndmin=2)
        self.LoadWavefunctionData((r + 1j * c).reshape(tuple(self.psi.GetData().shape)))

    def LoadWavefunctionHDF(self, filename, datasetPath):
        raise NotImplementedError("HDF5 wavefunction files (serialization/WavefunctionHDF.py) need pytables or "
                                  "h5py; use WavefunctionFileFormat.Binary or Ascii")

    def SaveWavefunctionHDF(self, filename, datasetPath):
        self.LoadWavefunctionHDF(filename, datasetPath)

    def SetupWavefunctionFunction(self, config):
        """f(conf, [l, r]) on (l, radial quadrature points), projected onto the
        B-splines: c_l = S^-1 <B | f(l, .)>."""
        ic = config.InitialCondition
        repr_ = self.psi.GetRepresentation()
        bs = repr_.radial.bspline
        B, _, _ = bs.tables()
        ls = repr_.angular.lvalues()
        out = np.zeros(repr_.GetFullShape(), dtype=np.complex128)
        for a, l in enumerate(ls):
            f = np.array([ic.function(ic, [float(l), r]) for r in bs.grid], dtype=np.complex128)
            rhs = B @ (bs.grid_weights * f)
            out[a] = np.linalg.solve(repr_.radial.S, rhs)
        self.psi.SetData(out)


def LoadPropagator(path, device=None):
    """pyprop.LoadPropagator(config.ini) as the reference README describes it:
    Problem(Load(path))."""
    return Problem(Load(path), device=device)
