"""Representations and the wavefunction of a rank-2 (angular, radial) problem.

Mirrors the reference objects the propagation path touches:
  CombinedRepresentation<2>           core/representation/combinedrepresentation.{h,cpp}
  ReducedSphericalHarmonicRepresentation  core/representation/reducedspherical/reducedsphericalharmonicrepresentation.h:16-99
  BSplineRepresentation + OverlapMatrix    core/representation/bspline/, core/representation/overlapmatrix.cpp:9-104
  Wavefunction<2>                     core/wavefunction.{h,cpp} (C order psi[l][r], radial fastest)
Setup and observables only; the step itself runs in libgbprop.
"""
from __future__ import annotations

import numpy as np

from .basis import bspline as _bs
from .basis import sphharm as _sph


class ReducedSphericalHarmonicRepresentation:
    """Angular rank: l = |m|..maxl at fixed m; orthogonal, unit weights."""

    def __init__(self):
        self.tools = None

    def ApplyConfigSection(self, sec):
        self.SetupRepresentation(int(sec.maxl), int(getattr(sec, "m", 0)))

    def SetupRepresentation(self, lmax, m=0):
        self.tools = _sph.ReducedSphericalTools(lmax, m)

    @property
    def count(self):
        return self.tools.lmax + 1 - abs(self.tools.m)

    def lvalues(self):
        return self.tools.lvalues()

    def IsOrthogonalBasis(self):
        return True


class BSplineRepresentation:
    """Radial rank: B-spline basis with its overlap matrix S and Cholesky factor U (S = U^T U)."""

    def __init__(self):
        self.bspline = None

    def ApplyConfigSection(self, sec):
        self.SetupRepresentation(_bs.bspline_from_section(sec))

    def SetupRepresentation(self, bspline):
        self.bspline = bspline
        self.kd = bspline.order - 1
        self.S = bspline.overlap()
        self.U = _bs.band_cholesky_upper(self.S, self.kd)

    @property
    def count(self):
        return self.bspline.count

    def cholesky_band(self):
        """U in upper band storage (n, kd+1): U(i,j) at j*(kd+1) + kd + i - j
        (OverlapMatrix::OverlapCholeskyUpper, overlapmatrix.cpp:22-37)."""
        n, kd = self.count, self.kd
        out = np.zeros(n * (kd + 1))
        for j in range(n):
            for i in range(max(0, j - kd), j + 1):
                out[j * (kd + 1) + kd + i - j] = self.U[i, j]
        return out

    def overlap_diagonals(self):
        """S as (2kd+1, n) diagonals: S(i, i+d-kd) at [d, i] (zero outside)."""
        n, kd = self.count, self.kd
        D = np.zeros((2 * kd + 1, n))
        for d in range(-kd, kd + 1):
            i = np.arange(max(0, -d), min(n, n - d))
            D[d + kd, i] = self.S[i, i + d]
        return D

    def IsOrthogonalBasis(self):
        return False


class CombinedRepresentation:
    """Rank-2 combined representation: rank 0 angular, rank 1 radial."""

    def __init__(self, rank=2):
        if rank != 2:
            raise NotImplementedError("only rank-2 (angular, radial) problems are provided")
        self.rank = rank
        self.reprs = [None, None]

    def SetRepresentation(self, i, r):
        self.reprs[i] = r

    def GetRepresentation(self, i):
        return self.reprs[i]

    @property
    def angular(self):
        return self.reprs[0]

    @property
    def radial(self):
        return self.reprs[1]

    def GetFullShape(self):
        return (self.angular.count, self.radial.count)

    def IsOrthogonalBasis(self, i):
        return self.reprs[i].IsOrthogonalBasis()

    def ApplyConfigSection(self, sec):
        pass


# ---------------------------------------------------------------------------
# wavefunction
# ---------------------------------------------------------------------------
def _torch():
    import torch
    return torch


class Wavefunction:
    """psi[l][r] complex (complex128 for the FP64 path, complex64 for the mixed path).

    Data lives in a torch tensor on the CUDA device when one is present, so
    that the propagation kernels work on it in place."""

    def __init__(self, representation, dtype="complex128", device=None):
        torch = _torch()
        self.repr = representation
        self.dtype = getattr(torch, dtype) if isinstance(dtype, str) else dtype
        if device is None:
            device = "cuda" if torch.cuda.is_available() else "cpu"
        self.device = torch.device(device)
        self.data = torch.zeros(representation.GetFullShape(), dtype=self.dtype, device=self.device)
        self._handle = None             # libgbprop handle of this representation (set by SetupStep)

    def GetRank(self):
        return 2

    def GetRepresentation(self):
        return self.repr

    def GetData(self):
        return self.data

    def GetDataNumpy(self):
        return self.data.detach().to("cpu").numpy()

    def SetData(self, arr):
        torch = _torch()
        self.data.copy_(torch.as_tensor(np.asarray(arr)).to(self.data.dtype))

    def AttachHandle(self, handle):
        """Route InnerProduct / GetNorm / Normalize of device wavefunctions through the handle's
        kernels (gbprop_inner_product)."""
        self._handle = handle

    def Copy(self):
        w = Wavefunction.__new__(Wavefunction)
        w.repr, w.dtype, w.device = self.repr, self.dtype, self.device
        w.data = self.data.clone()
        w._handle = getattr(self, "_handle", None)
        return w

    CopyDeep = Copy

    def Clear(self):
        self.data.zero_()

    # S-metric inner products (CombinedRepresentation::InnerProduct, Algorithm 4:
    # combinedrepresentation.cpp:423-474 -- S along the B-spline rank, identity on l)
    def _apply_overlap(self, x):
        torch = _torch()
        D = torch.as_tensor(self.repr.radial.overlap_diagonals(), dtype=torch.float64, device=x.device)
        kd = self.repr.radial.kd
        n = x.shape[1]
        xd = x.to(torch.complex128)
        out = torch.zeros_like(xd)
        for d in range(-kd, kd + 1):
            lo, hi = max(0, -d), min(n, n - d)
            out[:, lo:hi] += D[d + kd, lo:hi] * xd[:, lo + d:hi + d]
        return out

    def InnerProduct(self, other):
        """<self|other> in the overlap metric.  Device wavefunctions with a handle: libgbprop
        (gbprop_inner_product); otherwise (host set-up, e.g. initial states) in torch."""
        h = getattr(self, "_handle", None)
        if h is not None and self.data.is_cuda and other.data.is_cuda and other.data.dtype == self.data.dtype:
            return h.inner_product(self.data, other.data)
        torch = _torch()
        So = self._apply_overlap(other.data)
        return complex(torch.sum(torch.conj(self.data.to(torch.complex128)) * So).item())

    def GetNorm(self):
        return float(np.sqrt(abs(self.InnerProduct(self))))

    def Normalize(self):
        n = self.GetNorm()
        if n > 0:
            self.data /= n
        return n
