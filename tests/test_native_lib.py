"""The C-ABI library: it loads and exports every symbol the header declares.
No compute calls here (they need a GPU)."""
import ctypes
import os

import pytest

from pyprop_gb300 import _native


def test_library_exports_header_symbols():
    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("libgbprop.so not built (run __graft_entry__.build())")
    L = ctypes.CDLL(_native.LIB_PATH)
    declared = _native.declared_symbols()
    assert len(declared) >= 15
    missing = [s for s in declared if not hasattr(L, s)]
    assert missing == []
    # every declared symbol has a ctypes prototype in the binding
    assert set(declared) <= set(_native._PROTOS)


def test_version_and_errors_without_device():
    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("libgbprop.so not built")
    L = _native.lib()
    assert L.gbprop_version().startswith(b"gbprop")
    # argument validation happens before any device call
    h = ctypes.c_void_p()
    st = L.gbprop_create(ctypes.byref(h), 0, 10, 0, 20, 0, 0, None)
    assert st == 1 and b"positive" in L.gbprop_last_error()
    st = L.gbprop_create(ctypes.byref(h), 4, 10, 0, 99, 0, 0, None)
    assert st == 1 and b"krylov_basis_size" in L.gbprop_last_error()
    st = L.gbprop_create(ctypes.byref(h), 4, 10, 0, 20, 2, 0, None)   # exponentiation methods are 0 and 1
    assert st == 1 and b"krylov_exponentiation_method" in L.gbprop_last_error()
    st = L.gbprop_tensor_multiply_bandnh(5, None, 0, None, 1, 1.0, None, None, 1, 1, None)
    assert st == 7
    st = L.gbprop_advance(None, None, 1, None, 0.1, 0.0)
    assert st == 1
    # the banded bound-state solver validates sizes and pointers before touching a device
    st = L.gbprop_bound_states(100, 9, 4, None, None, 0.0, 8, None, None, None, None)   # kd > 8
    assert st == 1 and b"sizes" in L.gbprop_last_error()
    st = L.gbprop_bound_states(100, 6, 4, None, None, 0.0, 8, None, None, None, None)
    assert st == 1 and b"null" in L.gbprop_last_error()


def test_product_fails_loudly_without_device(small_problem_cpu):
    # the propagation path has no CPU fallback
    with pytest.raises(RuntimeError):
        small_problem_cpu.Propagator.SetupStep(small_problem_cpu.TimeStep)
