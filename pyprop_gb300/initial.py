"""Initial states used by the workload configurations."""
from __future__ import annotations

import math

import numpy as np


def overlap_norm2_exact(c, D, kd):
    """c^H (I x S) c for coefficients c (nl, nr), S given by its band diagonals D (2kd+1, nr),
    D[kd + d, i] = S(i, i + d): the products are formed elementwise and summed by math.fsum,
    which rounds the exact sum once, so the value (and every state normalised with it) is the
    same on every host."""
    c = np.asarray(c, dtype=np.complex128)
    nr = c.shape[1]
    terms = []
    for d in range(-kd, kd + 1):
        i = np.arange(max(0, -d), min(nr, nr - d))
        a, b = c[:, i], c[:, i + d]
        w = D[kd + d, i]
        terms.append((w * a.real * b.real).ravel())
        terms.append((w * a.imag * b.imag).ravel())
    return math.fsum(np.concatenate(terms).tolist())


def GaussianRandomState(psi, conf):
    """Seeded complex Gaussian coefficients, normalised in the overlap metric:
    psi^H (I x S) psi = 1 (the norm summed exactly, overlap_norm2_exact).  Section keys: `seed`."""
    seed = int(getattr(conf, "seed", 20261203))
    repr_ = psi.GetRepresentation()
    shape = repr_.GetFullShape()
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    rad = repr_.radial
    nrm = math.sqrt(overlap_norm2_exact(c, rad.overlap_diagonals(), rad.kd))
    # real divisions per component (complex division by a real differs between numpy builds)
    out = np.empty(shape, dtype=np.complex128)
    out.real = c.real / nrm
    out.imag = c.imag / nrm
    psi.SetData(out)
