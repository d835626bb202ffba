"""ctypes binding of libgbprop (include/gbprop.h).

The library is built in-tree by pyprop_gb300/csrc/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for the propagation path.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbprop.so")

GBPROP_OK = 0
STATUS_NAMES = {
    0: "GBPROP_OK", 1: "GBPROP_EINVAL", 2: "GBPROP_ECUDA", 3: "GBPROP_EBREAKDOWN",
    4: "GBPROP_ENONFINITE", 5: "GBPROP_ETIMEOUT", 6: "GBPROP_ELU", 7: "GBPROP_EUNSUPPORTED",
}
FP64 = 0
FP32_MIXED = 1
STORAGE_DIAG = 0
STORAGE_IDENT = 1
STORAGE_SIMP = 2
DEBUG_WAIT_LIMIT = 0
DEBUG_INJECT_LU = 1
DEBUG_ROUND_MATVEC = 2


class GbpropError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class Stats(C.Structure):
    _fields_ = [
        ("operator_count", C.c_longlong),
        ("inner_product_count", C.c_longlong),
        ("orthogonalization_count", C.c_longlong),
        ("breakdown_count", C.c_longlong),
        ("step_count", C.c_longlong),
        ("last_basis_size", C.c_int),
        ("last_scaling_order", C.c_int),
        ("error_estimate", C.c_double),
    ]


class ExpokitStats(C.Structure):
    _fields_ = [
        ("substeps", C.c_longlong),
        ("rejections", C.c_longlong),
        ("matvecs", C.c_longlong),
        ("error", C.c_double),
        ("hump", C.c_double),
        ("last_step", C.c_double),
    ]


PHASES = ["solve", "band", "gram_schmidt", "exponential", "combine", "other"]


class StepTimers(C.Structure):
    _fields_ = [
        ("ms", C.c_double * 6),
        ("count", C.c_int * 6),
        ("total_ms", C.c_double),
        ("launches", C.c_longlong),
    ]


_lib = None

# name -> (restype, argtypes)
_PROTOS = {
    "gbprop_version": (C.c_char_p, []),
    "gbprop_last_error": (C.c_char_p, []),
    "gbprop_launch_count": (C.c_longlong, []),
    "gbprop_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "gbprop_destroy": (C.c_int, [C.c_void_p]),
    "gbprop_set_overlap": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "gbprop_add_potential": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "gbprop_finalize": (C.c_int, [C.c_void_p]),
    "gbprop_advance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_double]),
    "gbprop_advance_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_double]),
    "gbprop_matvec": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]),
    "gbprop_matvec_scalings": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "gbprop_multiply_sqrt_overlap": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbprop_set_renormalization": (C.c_int, [C.c_void_p, C.c_int]),
    "gbprop_inner_product": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbprop_solve_sqrt_overlap": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "gbprop_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "gbprop_reset_stats": (C.c_int, [C.c_void_p]),
    "gbprop_get_hessenberg": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbprop_synchronize": (C.c_int, [C.c_void_p]),
    "gbprop_debug_set": (C.c_int, [C.c_void_p, C.c_int, C.c_longlong]),
    "gbprop_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_void_p]),
    "gbprop_bound_states": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbprop_debug_expm": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p,
                                    C.POINTER(C.c_int)]),
    "gbprop_time_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                   C.POINTER(StepTimers)]),
    "gbprop_tensor_multiply_bandnh": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_double,
                                                C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "gbprop_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "gbprop_expokit_advance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.POINTER(ExpokitStats)]),
    "gbprop_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_void_p]),
    "gbprop_batch_advance": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.c_void_p]),
    "gbprop_batch_destroy": (C.c_int, [C.c_void_p]),
    "gbprop_batch_synchronize": (C.c_int, [C.c_void_p]),
    "gbprop_block_inner_product_workspace": (C.c_size_t, [C.c_long, C.c_int]),
    "gbprop_block_inner_product": (C.c_int, [C.c_int, C.c_void_p, C.c_long, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                             C.c_void_p, C.c_size_t, C.c_void_p]),
    "gbprop_bspline_bands": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    "gbprop_block_inner_product_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_long, C.c_int, C.c_void_p, C.c_int,
                                                     C.c_void_p, C.c_void_p]),
}


def declared_symbols():
    """Every extern "C" function name declared in include/gbprop.h."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "gbprop.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(gbprop_[a-z_0-9]+)\s*\(", text)))


def lib():
    """Load libgbprop.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libgbprop.so not built (run pyprop_gb300/csrc/build.py or __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status):
    if status != GBPROP_OK:
        msg = lib().gbprop_last_error()
        raise GbpropError(status, msg.decode() if msg else "")
    return status


def ptr(x):
    """Device or host address of a torch tensor / numpy array, or None."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    if hasattr(x, "ctypes"):
        return C.c_void_p(x.ctypes.data)
    return C.c_void_p(int(x))


class Handle:
    """Owning wrapper of a gbprop_handle."""

    def __init__(self, nl, nr, precision=FP64, krylov_basis_size=20, exponentiation_method=0,
                 double_orthogonalization=False, stream=None):
        L = lib()
        h = C.c_void_p()
        check(L.gbprop_create(C.byref(h), int(nl), int(nr), int(precision), int(krylov_basis_size),
                              int(exponentiation_method), int(bool(double_orthogonalization)),
                              C.c_void_p(stream or 0)))
        self._h = h
        self.nl, self.nr, self.precision, self.m = nl, nr, precision, krylov_basis_size
        self.nfuncs = 1                 # time functions (the largest number given to add_potential)

    def __del__(self):
        try:
            if getattr(self, "_h", None) and self._h.value:
                lib().gbprop_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    @property
    def raw(self):
        return self._h

    def set_overlap(self, kd, U_band):
        import numpy as np
        U = np.ascontiguousarray(U_band, dtype=np.float64)
        check(lib().gbprop_set_overlap(self._h, int(kd), ptr(U)))

    def add_potential(self, storage, pairs, kb, data, time_dependent):
        import numpy as np
        d = np.ascontiguousarray(data, dtype=np.complex128)
        npairs = d.shape[0]
        p = None
        if pairs is not None:
            p = np.ascontiguousarray(pairs, dtype=np.int32)
        k = int(time_dependent)        # False/True or a time-function number
        check(lib().gbprop_add_potential(self._h, int(storage), int(npairs), ptr(p), int(kb), ptr(d), k))
        self.nfuncs = max(self.nfuncs, k)

    def finalize(self):
        check(lib().gbprop_finalize(self._h))

    def _steps(self, scalings):
        """(nsteps, K) step-major time-function values: one value per step, or K per step."""
        import numpy as np
        s = np.asarray(scalings, dtype=np.float64)
        if s.ndim <= 1 and self.nfuncs == 1:
            s = s.reshape(-1, 1)
        s = np.ascontiguousarray(s.reshape(-1, self.nfuncs))
        return s

    def advance(self, psi_dev, scalings, dt):
        s = self._steps(scalings)
        dt = complex(dt)
        check(lib().gbprop_advance(self._h, ptr(psi_dev), int(s.shape[0]), ptr(s), dt.real, dt.imag))

    def advance_host(self, psi_host, scalings, dt):
        s = self._steps(scalings)
        dt = complex(dt)
        check(lib().gbprop_advance_host(self._h, ptr(psi_host), int(s.shape[0]), ptr(s), dt.real, dt.imag))

    def matvec(self, src, dst, scaling, balanced=True):
        """dst = (balanced) operator at time-function value(s) `scaling`: one value for every
        time function, or K values."""
        import numpy as np
        v = np.asarray(scaling, dtype=np.float64).reshape(-1)
        if v.size == 1:
            check(lib().gbprop_matvec(self._h, ptr(src), ptr(dst), float(v[0]), int(bool(balanced))))
        else:
            v = np.ascontiguousarray(v)
            check(lib().gbprop_matvec_scalings(self._h, ptr(src), ptr(dst), ptr(v), int(bool(balanced))))

    def set_renormalization(self, on):
        """Every step ends with psi <- psi / ||psi||_S (Problem.py:167-168), on the device."""
        check(lib().gbprop_set_renormalization(self._h, int(bool(on))))

    def inner_product(self, a, b):
        """a^H (I x S) b of two device wavefunctions (synchronous)."""
        out = (C.c_double * 2)()
        check(lib().gbprop_inner_product(self._h, ptr(a), ptr(b), out))
        return complex(out[0], out[1])

    def multiply_sqrt_overlap(self, psi):
        check(lib().gbprop_multiply_sqrt_overlap(self._h, ptr(psi)))

    def solve_sqrt_overlap(self, conj, psi):
        check(lib().gbprop_solve_sqrt_overlap(self._h, int(bool(conj)), ptr(psi)))

    def stats(self):
        st = Stats()
        check(lib().gbprop_get_stats(self._h, C.byref(st)))
        return st

    def reset_stats(self):
        check(lib().gbprop_reset_stats(self._h))

    def tuning(self):
        """(band-kernel variant, (U^-1 solve chunks, U^-T solve chunks)) chosen by the autotuner."""
        import numpy as np
        v = C.c_int()
        ch = np.zeros(2, dtype=np.int32)
        check(lib().gbprop_get_tuning(self._h, C.byref(v), ch.ctypes.data))
        return v.value, (int(ch[0]), int(ch[1]))

    def hessenberg(self):
        import numpy as np
        out = np.zeros((self.m, self.m), dtype=np.complex128)
        check(lib().gbprop_get_hessenberg(self._h, ptr(out)))
        return out

    def synchronize(self):
        """Wait for the handle's work; raises GbpropError for a device-side failure of it."""
        check(lib().gbprop_synchronize(self._h))

    def time_step(self, psi_dev, scaling, dt):
        """One step outside the graph with an event per launch; returns
        {phase: (ms, launches)}, plus 'total_ms' and 'launches'."""
        dt = complex(dt)
        t = StepTimers()
        s = self._steps(scaling)[:1]
        check(lib().gbprop_time_step(self._h, ptr(psi_dev), ptr(s), dt.real, dt.imag, C.byref(t)))
        out = {name: (t.ms[k], t.count[k]) for k, name in enumerate(PHASES)}
        out["total_ms"] = t.total_ms
        out["launches"] = t.launches
        return out

    def debug_expm(self, H, dt, form):
        """y = exp(-i dt H) e1 by one of the handle's exponential kernels (0 FP64 Pade, 1 double-float
        Pade, 2 eigenvector) on a host Hessenberg matrix; returns (y, scaling order)."""
        import numpy as np
        Hc = np.ascontiguousarray(H, dtype=np.complex128)
        y = np.zeros(self.m, dtype=np.complex128)
        so = C.c_int()
        dt = complex(dt)
        check(lib().gbprop_debug_expm(self._h, ptr(Hc), dt.real, dt.imag, int(form), ptr(y), C.byref(so)))
        return y, so.value

    def debug_set(self, key, value):
        """Test hooks of the failure paths (DEBUG_WAIT_LIMIT, DEBUG_INJECT_LU; see gbprop.h)."""
        check(lib().gbprop_debug_set(self._h, int(key), int(value)))

    def expokit_advance(self, psi_dev, scalings, dt, tol, anorm):
        """Expokit steps (Krylov dimension = this handle's basis size - 1); returns ExpokitStats."""
        s = self._steps(scalings)
        dt = complex(dt)
        st = ExpokitStats()
        check(lib().gbprop_expokit_advance(self._h, ptr(psi_dev), int(s.shape[0]), ptr(s), dt.real, dt.imag,
                                           float(tol), float(anorm), C.byref(st)))
        return st

    def autotune(self, variant=-1):
        """Time the band kernel's tile shapes and keep the fastest (variant < 0), or select
        `variant`; returns the shape in use."""
        v = C.c_int(int(variant))
        check(lib().gbprop_autotune(self._h, C.byref(v)))
        return v.value


class Batch:
    """Owning wrapper of a gbprop_batch over finalized Handles (kept alive here)."""

    def __init__(self, handles, autotune=True, stream=None):
        L = lib()
        self.handles = list(handles)
        arr = (C.c_void_p * len(self.handles))(*[h.raw.value for h in self.handles])
        b = C.c_void_p()
        check(L.gbprop_batch_create(C.byref(b), arr, len(self.handles), int(bool(autotune)), C.c_void_p(stream or 0)))
        self._b = b

    def __del__(self):
        try:
            if getattr(self, "_b", None) and self._b.value:
                lib().gbprop_batch_destroy(self._b)
                self._b = C.c_void_p()
        except Exception:
            pass

    def advance(self, psis, scalings, dts):
        """psis: list of device tensors; scalings: per problem a (nsteps,) or (nsteps, K_p)
        array (a (count, nsteps) array when every problem has one time function); dts: complex
        per problem."""
        import numpy as np
        P = len(self.handles)
        blocks = [h._steps(scalings[p]) for p, h in enumerate(self.handles)]
        nsteps = blocks[0].shape[0]
        if any(b.shape[0] != nsteps for b in blocks):
            raise ValueError("every problem of a batch advances the same number of steps")
        s = np.ascontiguousarray(np.concatenate([b.reshape(-1) for b in blocks]))
        d = np.ascontiguousarray(np.array([[complex(x).real, complex(x).imag] for x in dts], dtype=np.float64))
        arr = (C.c_void_p * P)(*[p.data_ptr() for p in psis])
        check(lib().gbprop_batch_advance(self._b, arr, int(nsteps), ptr(s), ptr(d)))

    def synchronize(self):
        """Wait for the batch; raises GbpropError for a device-side failure of any member."""
        check(lib().gbprop_batch_synchronize(self._b))


def block_inner_product(V, w, want_norm=False, stream=None):
    """conj(V) @ w for the rows of a device matrix V (nv <= 45 rows of n elements, complex128 or
    complex64, like w) through gbprop_block_inner_product; with want_norm, ||w||^2 as well.
    Returns a device float64 tensor: 2 nv values (re, im interleaved) [+ ||w||^2]."""
    import torch
    nv, n = V.shape[0], w.numel()
    prec = FP64 if V.dtype == torch.complex128 else FP32_MIXED
    L = lib()
    ws = int(L.gbprop_block_inner_product_workspace(n, nv))
    work = torch.empty(ws, dtype=torch.uint8, device=V.device)
    out = torch.empty(2 * nv + (1 if want_norm else 0), dtype=torch.float64, device=V.device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(L.gbprop_block_inner_product(prec, ptr(V), n, nv, ptr(w), int(bool(want_norm)), ptr(out), ptr(work), ws,
                                       C.c_void_p(st)))
    return out


RADIAL_CONST, RADIAL_INV_R, RADIAL_INV_2R2 = 0, 1, 2


def bspline_bands(bspline, terms, cholesky=False, stream=None):
    """Band matrices <B_i| f |d^n B_j> of a basis.bspline.BSplineBasis on the GPU
    (gbprop_bspline_bands).  terms: list of (function id, derivative order, coefficient) with
    f = c, c / r or c / (2 r^2) (RADIAL_CONST, RADIAL_INV_R, RADIAL_INV_2R2).  Returns the list of
    (2k - 1, n) diagonal arrays (D[k - 1 + d, i] = M(i, i + d), as BSplineBasis.band_diagonals)
    and, with cholesky, the (k, n) upper Cholesky diagonals of the first matrix."""
    import numpy as np
    k, n = bspline.order, bspline.count
    knots = np.ascontiguousarray(bspline.knots, dtype=np.float64)
    bps = np.ascontiguousarray(bspline.breakpoints, dtype=np.float64)
    nodes = np.ascontiguousarray(bspline.nodes, dtype=np.float64)
    wts = np.ascontiguousarray(bspline.weights, dtype=np.float64)
    fid = np.ascontiguousarray([t[0] for t in terms], dtype=np.int32)
    der = np.ascontiguousarray([t[1] for t in terms], dtype=np.int32)
    coef = np.ascontiguousarray([t[2] for t in terms], dtype=np.float64)
    out = np.zeros((len(terms), 2 * k - 1, n))
    ch = np.zeros((k, n)) if cholesky else None
    check(lib().gbprop_bspline_bands(k, len(knots), ptr(knots), len(bps), ptr(bps), len(nodes), ptr(nodes), ptr(wts),
                                     len(terms), ptr(fid), ptr(der), ptr(coef), ptr(out), ptr(ch),
                                     C.c_void_p(stream or 0)))
    return [out[m] for m in range(len(terms))], ch


def bound_states(h_bands, s_band, emax=0.0, max_states=64, stream=None):
    """gbprop_bound_states: h_bands (nrows, 2kd+1, nr) and s_band (2kd+1, nr) float64 CUDA tensors
    (symmetric bands, diagonal-major).  Returns (counts (nrows,) numpy, energies (nrows,
    max_states) numpy, vectors (nrows, max_states, nr) float64 CUDA tensor)."""
    import numpy as np
    import torch
    nrows, W, nr = h_bands.shape
    kd = (W - 1) // 2
    hb = h_bands.contiguous()
    sb = s_band.contiguous()
    counts = np.zeros(nrows, dtype=np.int32)
    energies = np.zeros((nrows, max_states), dtype=np.float64)
    vectors = torch.zeros((nrows, max_states, nr), dtype=torch.float64, device=hb.device)
    st = torch.cuda.current_stream(hb.device).cuda_stream if stream is None else stream
    check(lib().gbprop_bound_states(nr, kd, nrows, ptr(hb), ptr(sb), float(emax), int(max_states), ptr(counts),
                                    ptr(energies), ptr(vectors), C.c_void_p(st)))
    return counts, energies, vectors


def launch_count():
    return int(lib().gbprop_launch_count())
