"""TensorPotential generation and consolidation (setup, host side).

Produces each potential in the reference's own storage so that it can be
handed to libgbprop exactly as the reference hands PotentialData to its
generated kernels:
  TensorPotential               pyprop/tensorpotential/TensorPotential.py:3-163
  GeometryInfo storages         pyprop/tensorpotential/GeometryInfo.py:240-285 (Diag),
                                :407-459 (BandNH), basis/ReducedSphericalHarmonic.py:5-45 (Simp)
  TensorPotentialGenerator      pyprop/tensorpotential/TensorPotentialGenerator.py:72-256
                                (evaluate on the tensor grid, project rank by rank, last rank first)
  BasisPropagator potential list / consolidation
                                pyprop/tensorpotential/BasisPropagator.py:41-108
"""
from __future__ import annotations

import numpy as np

from . import potentials as _pot
from .basis import sphharm as _sph


class GeometryInfo:
    """Storage of one rank of a TensorPotential."""

    def __init__(self, storage_id, pairs, count, use_grid, band_count=None):
        self.storage_id = storage_id
        self._pairs = pairs
        self.count = count
        self.use_grid = use_grid
        self.band_count = band_count

    def GetStorageId(self):
        return self.storage_id

    def GetBasisPairs(self):
        return self._pairs

    def GetGlobalBasisPairCount(self):
        return self.count

    def UseGridRepresentation(self):
        return self.use_grid


def bandnh_pairs(n, k):
    """GeometryInfoCommonBandedNonHermitian.GetBasisPairs (GeometryInfo.py:433-454):
    slot j*(2k+1) + k + i - j holds (i, j); unused slots default to (0, n-1)."""
    W = 2 * k + 1
    pairs = np.zeros((n * W, 2), dtype=np.int32)
    pairs[:, 1] = n - 1
    for i in range(n):
        for j in range(max(0, i - k), min(n, i + k + 1)):
            idx = j * W + k + i - j
            pairs[idx, 0] = i
            pairs[idx, 1] = j
    return pairs


def dense_to_bandnh(M, k):
    """Dense n x n band matrix -> BandNH storage (n*(2k+1),): element (i,j) at j*(2k+1)+k+i-j."""
    n = M.shape[0]
    W = 2 * k + 1
    out = np.zeros(n * W, dtype=np.result_type(M.dtype, np.complex128))
    for d in range(-k, k + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        j = i + d
        out[j * W + k + i - j] = M[i, j]
    return out


def diagonals_to_bandnh(D, kb):
    """Diagonals D[kb + d, i] = M(i, i+d) -> BandNH storage, (i, j) at j*(2kb+1) + kb + i - j."""
    n = D.shape[1]
    W = 2 * kb + 1
    out = np.zeros(n * W, dtype=np.result_type(D.dtype, np.complex128))
    for d in range(-kb, kb + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        out[(i + d) * W + kb - d] = D[kb + d, i]
    return out


def bandnh_to_dense(v, n, k):
    W = 2 * k + 1
    M = np.zeros((n, n), dtype=v.dtype)
    for d in range(-k, k + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        j = i + d
        M[i, j] = v[j * W + k + i - j]
    return M


class TensorPotential:
    """A potential expressed in the basis of a rank-2 (angular, radial) wavefunction."""

    def __init__(self, psi):
        self.psi = psi
        self.GeometryList = None
        self.PotentialData = None
        self.Name = None
        self.IsTimeDependent = False
        self.DebugPotential = False
        self.OriginalTimeFunction = None

    # TensorPotential.ApplyConfigSection (TensorPotential.py:33-78)
    def ApplyConfigSection(self, sec):
        self.DebugPotential = bool(getattr(sec, "debug_potential", False))
        self.IsTimeDependent = False
        if hasattr(sec, "time_function"):
            self.IsTimeDependent = True
            self.TimeFunction = lambda t, _s=sec: sec.time_function(_s, t)
            self.OriginalTimeFunction = sec.time_function
        self.Name = sec.name
        self.GeometryList = self._geometry(sec)
        self.PotentialData = self._generate(sec)

    def _geometry(self, sec):
        repr_ = self.psi.GetRepresentation()
        ang, rad = repr_.angular, repr_.radial
        g0 = sec.geometry0.lower().strip()
        use_grid0 = True
        if g0.startswith("custom-"):
            use_grid0 = False
            g0 = g0[len("custom-"):]
        if g0 == "diagonal":
            nl = ang.count
            geom0 = GeometryInfo("Diag", np.stack([np.arange(nl), np.arange(nl)], 1).astype(np.int32), nl, False)
        elif g0 == "identity":
            geom0 = GeometryInfo("Ident", np.zeros((1, 2), dtype=np.int32), 1, use_grid0)
        elif g0 == "dipoleselectionrule":
            pairs = _sph.selection_rule_pairs(ang.tools)
            geom0 = GeometryInfo("Simp", pairs, len(pairs), use_grid0)
        else:
            raise NotImplementedError("angular geometry %r is not provided (Diagonal, Identity, "
                                      "DipoleSelectionRule)" % sec.geometry0)
        g1 = sec.geometry1.lower().strip()
        if g1 != "banded-nonhermitian":
            raise NotImplementedError("radial geometry %r is not provided (banded-nonhermitian)" % sec.geometry1)
        k = rad.bspline.order - 1
        geom1 = GeometryInfo("BandNH", bandnh_pairs(rad.count, k), rad.count * (2 * k + 1), True, band_count=k)
        return [geom0, geom1]

    # TensorPotentialGenerator.GeneratePotential (TensorPotentialGenerator.py:72-256)
    def _generate(self, sec):
        repr_ = self.psi.GetRepresentation()
        ang, rad = repr_.angular, repr_.radial
        geom0, geom1 = self.GeometryList
        diff0 = int(getattr(sec, "differentiation0", 0))
        diff1 = int(getattr(sec, "differentiation1", 0))
        k = geom1.band_count
        bs = rad.bspline
        rgrid = bs.grid
        if geom0.storage_id == "Diag":
            agrid = ang.lvalues().astype(float)
        elif geom0.storage_id == "Ident":
            agrid = np.array([ang.lvalues()[0] if not geom0.use_grid else ang.tools.theta[0]], dtype=float)
        else:
            agrid = ang.tools.theta
        V = _pot.evaluate(sec, agrid, rgrid)              # (nang, nrgrid)
        # radial rank first (ranks are projected last to first)
        radial = np.zeros((len(agrid), rad.count * (2 * k + 1)), dtype=np.complex128)
        for a in range(len(agrid)):
            radial[a] = diagonals_to_bandnh(bs.band_diagonals(V[a], diff1), k)
        if geom0.storage_id == "Simp":
            data = _sph.project_angular(ang.tools, radial, geom0.GetBasisPairs(), diff0)
        else:
            if diff0 != 0:
                raise ValueError("differentiation0 requires a grid angular geometry")
            data = radial
        return np.ascontiguousarray(data, dtype=np.complex128)

    # TensorPotential.CanConsolidate (TensorPotential.py:128-163)
    def CanConsolidate(self, other):
        if self.IsTimeDependent != other.IsTimeDependent:
            return False
        if self.IsTimeDependent and other.IsTimeDependent and other.OriginalTimeFunction is not self.OriginalTimeFunction:
            return False
        if self.DebugPotential or other.DebugPotential:
            return False
        for a, b in zip(self.GeometryList, other.GeometryList):
            if a.GetStorageId() != b.GetStorageId():
                return False
        for a, b in zip(self.GeometryList, other.GeometryList):
            pa, pb = a.GetBasisPairs(), b.GetBasisPairs()
            if pa.shape != pb.shape or np.any(pa != pb):
                return False
        return True

    def GetStorageIds(self):
        return [g.GetStorageId() for g in self.GeometryList]

    def GetScaling(self, t):
        return float(self.TimeFunction(t)) if self.IsTimeDependent else 1.0


def generate_potentials(psi, config, names):
    """BasisPropagator.GeneratePotentials + ConsolidatePotentials
    (BasisPropagator.py:41-108): generate each listed potential, add it to an
    existing compatible one when possible, then consolidate the list."""
    potentials = []
    for name in names:
        sec = config.GetSection(name)
        pot = TensorPotential(psi)
        pot.ApplyConfigSection(sec)
        for existing in potentials:
            if existing.CanConsolidate(pot):
                existing.PotentialData = existing.PotentialData + pot.PotentialData
                existing.Name += "+" + pot.Name
                pot = None
                break
        if pot is not None:
            potentials.append(pot)
    i = 0
    while i < len(potentials) - 1:
        cur = potentials[i]
        for other in list(potentials[i + 1:]):
            if cur.CanConsolidate(other):
                cur.PotentialData = cur.PotentialData + other.PotentialData
                cur.Name += "+" + other.Name
                potentials.remove(other)
        i += 1
    return potentials
