"""Comparison of the sum columns of two FP32 observation rows (or averages)
whose fields are bit-identical but whose kernels add the per-site terms
differently.

The moment columns (phi2, pi2, phipi, phi4, phi6) agree to 1e-6 relative.
Energy, interaction and charge are sums of per-site terms that cancel: in the
tilted double well the interaction is -0.06 while its terms are of the size of
<phi^2>.  One kernel adds FP32 per-site terms, the x4 kernel forms the same
sums from FP64 moment totals, so the two differ by the FP32 rounding of those
terms: they are compared within 1e-7 of the row's quadratic scale
max(|<phi^2>|, |<pi^2>|) (FP32's unit roundoff is 6e-8), plus 1e-6 relative.
"""
from __future__ import annotations

import numpy as np

MOMENTS = slice(9, 14)     # phi2, pi2, phipi, phi4, phi6
ENERGIES = slice(14, 17)   # energy, interaction, charge
PHI2, PI2 = 9, 10


def assert_fp32_sums_close(a, b):
    a = np.atleast_2d(np.asarray(a, dtype=np.float64))
    b = np.atleast_2d(np.asarray(b, dtype=np.float64))
    assert a.shape == b.shape
    np.testing.assert_allclose(a[:, MOMENTS], b[:, MOMENTS], rtol=1e-6, atol=1e-9)
    scale = np.maximum(np.abs(b[:, PHI2]), np.abs(b[:, PI2]))[:, None]
    err = np.abs(a[:, ENERGIES] - b[:, ENERGIES])
    bound = 1e-7 * scale + 1e-6 * np.abs(b[:, ENERGIES])
    assert np.all(err <= bound), f"energy columns differ by {err.max():.3e} (bound {bound.min():.3e})"
