"""B-spline radial basis: breakpoints, knots, Gauss-Legendre quadrature and
overlap/differentiation integrals, following pyprop's B-spline setup.

Setup only (not on the timed path).  Everything here runs once per problem on
the host and produces the radial band matrices that the TensorPotential
assembly stores.

Reference behaviour restated:
  breakpoint sequences      pyprop/bspline/breakpointsequences.py:7-90
  continuity/knot sequence  pyprop/bspline/BSpline.py:93-161
  number of B-splines       pyprop/bspline/BSpline.py:30-33
  Gauss-Legendre rule       pyprop/bspline/gausslegendrequadrature.py:18-42 (Golub-Welsch)
  global quadrature grid    pyprop/bspline/BSpline.py:183-235, ScaleAndTranslate
                            core/transform/bspline/bspline.h:173-176
  B-spline recursion        core/transform/bspline/bspline.cpp:26-164 (eps = 1e-15, bspline.h:58)
  overlap integral          core/transform/bspline/bspline.cpp:373-467 (swap i>j => factor (-1)^n)
"""
from __future__ import annotations

import math
import numpy as np

EPS = 1e-15


# --------------------------------------------------------------------------
# breakpoint sequences
# --------------------------------------------------------------------------
def linear_breakpoints(rmin, rmax, n):
    """LinearBreakpointSequence (breakpointsequences.py:31-38)."""
    return np.array([rmin + (rmax - rmin) * i / float(n - 1) for i in range(n)])


def exponential_breakpoints(rmin, rmax, n, gamma):
    """ExponentialBreakpointSequence (breakpointsequences.py:7-28)."""
    h = rmax - rmin
    return np.array([rmin + h * (math.exp(gamma * float(i - 1) / float(n - 1)) - 1.0) / (math.exp(gamma) - 1.0)
                     for i in range(1, n + 1)])


def _frange(xini, xfin, delta):
    """matplotlib.mlab.frange(xini, xfin, delta) with closed=1 (matplotlib <= 2.x):
    npts = int(round((xfin - xini) / delta)) + 1, values xini + k*delta."""
    npts = int(np.round((xfin - xini) / delta)) + 1
    return np.arange(npts) * delta + xini


def exponential_linear_breakpoints(rmin, rpartition, rmax, n, gamma):
    """ExponentialLinearBreakpointSequence (breakpointsequences.py:70-88): n exponential
    points on [rmin, rpartition], then linear spacing equal to the last exponential gap."""
    h = rpartition - rmin
    xi = [rmin + h * (math.exp(gamma * float(i - 1) / float(n - 1)) - 1.0) / (math.exp(gamma) - 1.0)
          for i in range(1, n + 1)]
    h = xi[-1] - xi[-2]
    xi += list(_frange(rpartition + h, rmax, h))
    return np.array(xi)


def make_breakpoints(bpstype, xmin, xmax, xsize, gamma=None, xpartition=None):
    """BSPLINE.CreateBreakpointSequence (BSpline.py:46-90) for the supported types."""
    if bpstype == "linear":
        return linear_breakpoints(xmin, xmax, xsize)
    if bpstype == "exponential":
        return exponential_breakpoints(xmin, xmax, xsize, gamma)
    if bpstype == "exponentiallinear":
        return exponential_linear_breakpoints(xmin, xpartition, xmax, xsize, gamma)
    raise NameError("Sequence not recognized: %r" % (bpstype,))


def continuity_sequence(nbreak, order, continuity, left=None, right=None):
    """BSPLINE.CreateContinuitySequence (BSpline.py:93-127)."""
    seq = (order - 1) * np.ones(nbreak, dtype=int)
    if continuity == "vanilla":
        seq[0] = 0
        seq[-1] = 0
    elif continuity == "zero":
        seq[0] = 1
        seq[-1] = 1
    elif continuity == "custom":
        seq[0] = left
        seq[-1] = right
    else:
        raise Exception("Unknown continuity type!")
    return seq


def knot_sequence(breakpoints, continuity, order):
    """BSPLINE.CreateKnotSequence (BSpline.py:133-161): breakpoint i repeated
    order - continuity[i] times."""
    knots = []
    for i, bp in enumerate(breakpoints):
        knots += [bp] * int(order - continuity[i])
    return np.array(knots, dtype=float)


def gauss_legendre(order):
    """GaussQuadratureRule (gausslegendrequadrature.py:18-42): Golub-Welsch on the
    symmetric tridiagonal Jacobi matrix of the Legendre recurrence."""
    if order == 1:
        return np.array([0.0]), np.array([2.0])
    beta = np.array([1.0 / (2.0 * math.sqrt(1.0 - (2.0 * n) ** -2)) for n in range(1, order)])
    J = np.diag(beta, -1) + np.diag(beta, 1)
    E, V = np.linalg.eigh(J)
    idx = np.argsort(E)
    return E[idx], 2.0 * V[0, idx] ** 2


_GL = {}


def _gauss_legendre_cached(order):
    if order not in _GL:
        _GL[order] = gauss_legendre(order)
    return _GL[order]


def scale_and_translate(x, a, b):
    """bspline.h:173-176: map [-1, 1] onto [a, b]."""
    return (x - 1.0) * (b - a) / 2.0 + b


class BSplineBasis:
    """Radial B-spline basis of order k on a breakpoint sequence.

    Attributes mirror the reference object: ``breakpoints``, ``continuity``,
    ``knots``, ``order`` (MaxSplineOrder), ``count`` (NumberOfBSplines),
    ``nodes``/``weights`` (reference quadrature rule), ``grid``/``grid_weights``
    (QuadratureGridGlobal / QuadratureWeightsGlobal).
    """

    def __init__(self, breakpoints, order, continuity, quad_order_additional=0):
        self.breakpoints = np.asarray(breakpoints, dtype=float)
        self.order = int(order)
        self.continuity = np.asarray(continuity, dtype=int)
        self.knots = knot_sequence(self.breakpoints, self.continuity, self.order)
        self.count = len(self.knots) - self.order
        self.nodes, self.weights = _gauss_legendre_cached(self.order + int(quad_order_additional))
        # every interval's points in order (the same operations as scale_and_translate, per element)
        a = self.breakpoints[:-1, None]
        b = self.breakpoints[1:, None]
        self.grid = ((self.nodes[None, :] - 1.0) * (b - a) / 2.0 + b).ravel()
        self.grid_weights = ((b - a) / 2.0 * self.weights[None, :]).ravel()
        self._tables = None

    # -- evaluation (bspline.cpp:26-164) ---------------------------------
    def _levels(self, x, kmax):
        """All B-splines of orders 1..kmax at points x, by the three-point
        recursion with the reference's `> eps` guards, evaluated for every
        spline index at once.  Returns a list indexed by order."""
        t = self.knots
        nk = len(t)
        x = np.asarray(x, dtype=float)
        out = [None]
        b = ((t[:-1, None] <= x[None, :]) & (x[None, :] < t[1:, None])).astype(float)
        out.append(b)
        with np.errstate(divide="ignore", invalid="ignore"):
            for k in range(2, kmax + 1):
                ni = nk - k
                prev = out[k - 1]
                i = np.arange(ni)
                d0 = (t[i + k - 1] - t[i])[:, None]
                d1 = (t[i + k] - t[i + 1])[:, None]
                b0 = prev[:ni]
                b1 = prev[1:ni + 1]
                term0 = np.where(b0 > EPS, (x[None, :] - t[i][:, None]) / d0 * b0, 0.0)
                term1 = np.where(b1 > EPS, (t[i + k][:, None] - x[None, :]) / d1 * b1, 0.0)
                out.append(term0 + term1)
        return out

    def local_tables(self):
        """Values of the `order` B-splines that can be non-zero at each quadrature point:
        first[g] = index of the first of them; (B, dB, d2B)[g, a] for spline first[g] + a.
        Same three-point recursions and `> eps` guards as the reference (bspline.cpp:26-164),
        evaluated only on each point's knot span."""
        if getattr(self, "_local", None) is not None:
            return self._local
        t0 = self.knots
        k = self.order
        x = self.grid
        ng = len(x)
        mu = np.searchsorted(t0, x, side="right") - 1
        # pad the knot sequence so that splines that do not exist near the ends (removed by
        # the continuity conditions) can be evaluated and then discarded; index t[i] -> tp[i + k]
        tp = np.concatenate([np.full(k, t0[0]), t0, np.full(k, t0[-1])])

        class _T:
            def __getitem__(self, idx):
                return tp[np.asarray(idx) + k]

        t = _T()
        levels = [None, np.ones((ng, 1))]
        with np.errstate(divide="ignore", invalid="ignore"):
            for q in range(2, k + 1):
                prev = levels[q - 1]
                cur = np.zeros((ng, q))
                for a in range(q):
                    i = mu - q + 1 + a
                    if a >= 1:
                        b0 = prev[:, a - 1]
                        d0 = t[i + q - 1] - t[i]
                        cur[:, a] += np.where(b0 > EPS, (x - t[i]) / d0 * b0, 0.0)
                    if a <= q - 2:
                        b1 = prev[:, a]
                        d1 = t[i + q] - t[i + 1]
                        cur[:, a] += np.where(b1 > EPS, (t[i + q] - x) / d1 * b1, 0.0)
                levels.append(cur)
            B = levels[k]
            D1 = np.zeros((ng, k))
            D2 = np.zeros((ng, k))
            for a in range(k):
                i = mu - k + 1 + a
                if a >= 1:
                    p1 = levels[k - 1][:, a - 1]
                    D1[:, a] += np.where(p1 > EPS, (k - 1.0) / (t[i + k - 1] - t[i]) * p1, 0.0)
                if a <= k - 2:
                    p2 = levels[k - 1][:, a]
                    D1[:, a] -= np.where(p2 > EPS, (k - 1.0) / (t[i + k] - t[i + 1]) * p2, 0.0)
                if k > 2:
                    # B^{k-2}_{i}, _{i+1}, _{i+2} at local offsets a-2, a-1, a of level k-2
                    def lv(off):
                        return levels[k - 2][:, off] if 0 <= off <= k - 3 else np.zeros(ng)
                    q1, q2, q3 = lv(a - 2), lv(a - 1), lv(a)
                    q1 = np.where(q1 > EPS, q1 * ((k - 2.0) / (t[i + k - 2] - t[i])), q1)
                    q2 = np.where(q2 > EPS, q2 * ((k - 2.0) / (t[i + k - 1] - t[i + 1])), q2)
                    q3 = np.where(q3 > EPS, q3 * ((k - 2.0) / (t[i + k] - t[i + 2])), q3)
                    a_ = (k - 1.0) / (t[i + k - 1] - t[i])
                    d_ = (k - 1.0) / (t[i + k] - t[i + 1])
                    D2[:, a] += np.where((q1 > EPS) | (q2 > EPS), a_ * (q1 - q2), 0.0)
                    D2[:, a] -= np.where((q2 > EPS) | (q3 > EPS), d_ * (q2 - q3), 0.0)
        first = mu - k + 1
        # splines beyond the basis (index >= count) are zero by construction of the knot span
        self._local = (first, np.nan_to_num(B), np.nan_to_num(D1), np.nan_to_num(D2))
        return self._local

    def tables(self):
        """(B, dB, d2B) on the global quadrature grid, each (count, ngrid)
        (CreateBSplineTable / CreateBSplineDerivativeTable, bspline.cpp:169-289),
        with the first- and second-derivative recursions of bspline.cpp:82-164."""
        if self._tables is not None:
            return self._tables
        k = self.order
        n = self.count
        t = self.knots
        x = self.grid
        lv = self._levels(x, k)
        B = lv[k][:n].copy()
        i = np.arange(n)
        with np.errstate(divide="ignore", invalid="ignore"):
            # first derivative (bspline.cpp:82-106)
            p1, p2 = lv[k - 1][i], lv[k - 1][i + 1]
            D1 = np.where(p1 > EPS, (k - 1.0) / (t[i + k - 1] - t[i])[:, None] * p1, 0.0)
            D1 = D1 - np.where(p2 > EPS, (k - 1.0) / (t[i + k] - t[i + 1])[:, None] * p2, 0.0)
            # second derivative (bspline.cpp:112-164)
            if k > 2:
                q1, q2, q3 = lv[k - 2][i], lv[k - 2][i + 1], lv[k - 2][i + 2]
                q1 = np.where(q1 > EPS, q1 * ((k - 2.0) / (t[i + k - 2] - t[i]))[:, None], q1)
                q2 = np.where(q2 > EPS, q2 * ((k - 2.0) / (t[i + k - 1] - t[i + 1]))[:, None], q2)
                q3 = np.where(q3 > EPS, q3 * ((k - 2.0) / (t[i + k] - t[i + 2]))[:, None], q3)
                a_ = ((k - 1.0) / (t[i + k - 1] - t[i]))[:, None]
                d_ = ((k - 1.0) / (t[i + k] - t[i + 1]))[:, None]
                D2 = np.where((q1 > EPS) | (q2 > EPS), a_ * (q1 - q2), 0.0)
                D2 = D2 - np.where((q2 > EPS) | (q3 > EPS), d_ * (q2 - q3), 0.0)
            else:
                D2 = np.zeros_like(B)
        # grid window of each spline: the breakpoint intervals inside [t_i, t_{i+k}]
        nq = len(self.nodes)
        lo = np.searchsorted(self.breakpoints, t[i], side="left")
        hi = np.searchsorted(self.breakpoints, t[i + k], side="left")
        self._window = np.stack([lo * nq, hi * nq], axis=1)
        self._tables = (B, D1, D2)
        return self._tables

    # -- integrals ---------------------------------------------------------
    def integral(self, f_grid, derivative, i, j):
        """BSplineGlobalOverlapIntegral(f, n, i, j) (bspline.cpp:373-467):
        <B_i | f | d^n B_j> with the reference's swap rule: for i > j the
        indices are exchanged and the result multiplied by (-1)^n."""
        factor = 1.0
        if i > j:
            i, j = j, i
            factor = (-1.0) ** derivative
        if j - i >= self.order:
            return 0.0
        B, D1, D2 = self.tables()
        right = (B, D1, D2)[derivative]
        g0 = self._window[j, 0]
        g1 = self._window[i, 1]
        w = self.grid_weights[g0:g1]
        f = np.asarray(f_grid)[g0:g1]
        acc = 0.0
        for q in range(g1 - g0):
            acc += w[q] * f[q] * B[i, g0 + q] * right[j, g0 + q]
        return factor * acc

    def band_matrix(self, f_grid, derivative):
        """Dense (count x count) matrix of <B_i|f|d^n B_j> for |i-j| < order,
        with the reference's swap rule.  f_grid may be real or complex."""
        n = self.count
        k = self.order
        f = np.asarray(f_grid)
        M = np.zeros((n, n), dtype=np.result_type(f.dtype, np.float64))
        B, D1, D2 = self.tables()
        right = (B, D1, D2)[derivative]
        wf = self.grid_weights * f
        win = self._window
        sign = (-1.0) ** derivative
        for d in range(k):
            i = np.arange(n - d)
            j = i + d
            g0 = win[j, 0]
            g1 = win[i, 1]
            span = int((g1 - g0).max()) if len(i) else 0
            vals = np.zeros(len(i), dtype=M.dtype)
            for q in range(span):
                g = g0 + q
                ok = g < g1
                gg = np.where(ok, g, 0)
                vals = vals + np.where(ok, wf[gg] * B[i, gg] * right[j, gg], 0.0)
            M[i, j] = vals
            if d:
                M[j, i] = sign * vals
        return M

    def overlap(self):
        """Overlap matrix S_ij = <B_i|B_j> (BSpline::SetupOverlap, bspline.cpp:781-785)."""
        return self.band_matrix(np.ones_like(self.grid), 0)

    def band_diagonals(self, f_grid, derivative):
        """The matrix elements of band_matrix as diagonals: D[k + d, i] = M(i, i + d),
        d = -k..k (k = order - 1), accumulated from each quadrature point's k
        non-zero splines; the i > j part follows the reference's swap rule
        M(j, i) = (-1)^n M(i, j) (bspline.cpp:384-392)."""
        n = self.count
        k = self.order
        f = np.asarray(f_grid)
        dt = np.result_type(f.dtype, np.float64)
        D = np.zeros((2 * (k - 1) + 1, n), dtype=dt)
        first, B, D1, D2 = self.local_tables()
        right = (B, D1, D2)[derivative]
        wf = self.grid_weights * f
        sign = (-1.0) ** derivative
        for a in range(k):
            i = first + a
            ok_i = (i >= 0) & (i < n)
            for b in range(a, k):
                d = b - a
                j = i + d
                ok = ok_i & (j < n)
                vals = wf * B[:, a] * right[:, b]
                acc = np.zeros(n, dtype=dt)
                np.add.at(acc, i[ok], vals[ok])
                D[k - 1 + d] += acc
        for d in range(1, k):
            D[k - 1 - d, d:] = sign * D[k - 1 + d, : n - d]
        return D

def bspline_from_section(sec):
    """BSPLINE.ApplyConfigSection (BSpline.py:16-44) from a config section."""
    order = int(sec.order)
    bps = make_breakpoints(sec.bpstype, sec.xmin, sec.xmax, sec.xsize,
                           gamma=getattr(sec, "gamma", None), xpartition=getattr(sec, "xpartition", None))
    cont = continuity_sequence(len(bps), order, sec.continuity,
                               getattr(sec, "left_point_continuity", None),
                               getattr(sec, "right_point_continuity", None))
    return BSplineBasis(bps, order, cont, getattr(sec, "quad_order_additional", 0))


def band_cholesky_upper_diagonals(Sdiag, kd):
    """Upper Cholesky factor from the diagonals of a symmetric band matrix
    (Sdiag[kd + d, i] = S(i, i+d)); returns Ud[d, i] = U(i, i+d), d = 0..kd."""
    n = Sdiag.shape[1]
    Ud = np.zeros((kd + 1, n))
    for j in range(n):
        # column j of U: U(i, j) for i in [j-kd, j]
        d0 = Sdiag[kd, j]
        for t in range(1, min(kd, j) + 1):
            d0 -= Ud[t, j - t] ** 2
        if not d0 > 0:
            raise np.linalg.LinAlgError("overlap matrix not positive definite at %d" % j)
        d0 = math.sqrt(d0)
        Ud[0, j] = d0
        for dd in range(1, kd + 1):
            i = j + dd
            if i >= n:
                break
            sv = Sdiag[kd + dd, j]
            for t in range(1, kd + 1):
                r = j - t
                if r < 0 or i - r > kd:
                    continue
                sv -= Ud[t, r] * Ud[i - r, r]
            Ud[dd, j] = sv / d0
    return Ud


def band_cholesky_upper(S, kd):
    """Upper Cholesky factor U (S = U^T U) of a symmetric positive definite band
    matrix, returned dense.  Setup for the balanced-overlap transform
    (OverlapMatrix::Setup -> zpbtrf 'U', core/representation/overlapmatrix.cpp:35-37)."""
    n = S.shape[0]
    U = np.zeros_like(S, dtype=float)
    for j in range(n):
        k0 = max(0, j - kd)
        d = S[j, j] - np.dot(U[k0:j, j], U[k0:j, j])
        if not d > 0:
            raise np.linalg.LinAlgError("overlap matrix not positive definite at %d" % j)
        d = math.sqrt(d)
        U[j, j] = d
        for i in range(j + 1, min(n, j + kd + 1)):
            kk0 = max(k0, i - kd)
            U[j, i] = (S[j, i] - np.dot(U[kk0:j, j], U[kk0:j, i])) / d
    return U
