"""The allocation-free block inner product against the workspace version.

gbprop_block_inner_product_noalloc serves callers that cannot allocate device
memory when they need the Arnoldi inner products (e.g. from inside a memory
pool's callback, or a host that allows no allocation after start-up): its reduction
scratch is a fixed array inside the library instead of a caller workspace.
This file is collected last so that a failure here cannot hide any other
test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(prec, n, nv, seed):
    import torch
    rng = np.random.default_rng(seed)
    cdt = np.complex128 if prec == 0 else np.complex64
    V = (rng.standard_normal((nv, n)) + 1j * rng.standard_normal((nv, n))).astype(cdt)
    w = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(cdt)
    return torch.as_tensor(V).cuda(), torch.as_tensor(w).cuda()


@pytest.mark.parametrize("prec,n,nv", [(0, 64000, 30), (1, 64000, 30), (0, 1060, 1), (1, 7, 45)])
def test_noalloc_matches_workspace_entry_point_twice(prec, n, nv):
    import torch
    from pyprop_gb300 import _native
    L = _native.lib()
    ws_bytes = L.gbprop_block_inner_product_workspace(n, nv)
    work = torch.zeros(ws_bytes, dtype=torch.uint8, device="cuda")
    for call, want_norm in enumerate((1, 0)):
        # two calls in a row with different data: the shared scratch must not carry state over
        dV, dw = _setup(prec, n, nv, seed=1000 * call + nv)
        ref = torch.zeros(2 * nv + 1, dtype=torch.float64, device="cuda")
        got = torch.full((2 * nv + 1,), -7.0, dtype=torch.float64, device="cuda")
        _native.check(L.gbprop_block_inner_product(prec, _native.ptr(dV), n, nv, _native.ptr(dw), want_norm,
                                                   _native.ptr(ref), _native.ptr(work), ws_bytes, None))
        _native.check(L.gbprop_block_inner_product_noalloc(prec, _native.ptr(dV), n, nv, _native.ptr(dw), want_norm,
                                                           _native.ptr(got), None))
        torch.cuda.synchronize()
        k = 2 * nv + (1 if want_norm else 0)
        r, g = ref.cpu().numpy()[:k], got.cpu().numpy()[:k]
        assert np.linalg.norm(g - r) <= 1e-13 * np.linalg.norm(r)
        # and both against a host reference
        V = dV.cpu().numpy().astype(np.complex128)
        w = dw.cpu().numpy().astype(np.complex128)
        h = g[0:2 * nv:2] + 1j * g[1:2 * nv:2]
        want = V.conj() @ w
        assert np.linalg.norm(h - want) <= 1e-13 * np.linalg.norm(want)


def test_noalloc_rejects_oversized_requests():
    import torch
    from pyprop_gb300 import _native
    L = _native.lib()
    dV, dw = _setup(0, 16, 1, seed=3)
    out = torch.zeros(200, dtype=torch.float64, device="cuda")
    st = L.gbprop_block_inner_product_noalloc(0, _native.ptr(dV), 16, 46, _native.ptr(dw), 0, _native.ptr(out), None)
    assert st == 1 and b"nv" in L.gbprop_last_error()
    st = L.gbprop_block_inner_product_noalloc(0, _native.ptr(dV), 0, 1, _native.ptr(dw), 0, _native.ptr(out), None)
    assert st == 1
