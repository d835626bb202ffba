"""Initial states used by the workload configurations."""
from __future__ import annotations

import numpy as np


def GaussianRandomState(psi, conf):
    """Seeded complex Gaussian coefficients, normalised in the overlap metric:
    psi^H (I x S) psi = 1.  Section keys: `seed` (int)."""
    seed = int(getattr(conf, "seed", 20261203))
    shape = psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    psi.SetData(c)
    psi.Normalize()
