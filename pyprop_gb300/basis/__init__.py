"""Setup-time bases: radial B-splines and reduced spherical harmonics."""
