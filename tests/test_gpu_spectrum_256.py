"""The FP32 spectrum binning at 256^3 (bin_runs over a key table of the
reference's bins and of uniform bins) against the FP64 spectrum of the same
FP32-valued fields: mode counts exact; F and K (sums of positive terms)
within 1e-5 relative, Q within 1e-5 of the largest |Q| (the FP32
transform's rounding dominates; a mode binned wrongly moves a bin by far
more), for the reference bins and for 64 and 1024 uniform bins."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_fp32_binning_matches_fp64_at_256():
    from phinum_gb300 import lattice as PL
    N = 256
    phi, pi = inputs.lattice_fields(N, 1, seed=77)
    phi = phi.astype(np.float32).astype(np.float64)
    pi = pi.astype(np.float32).astype(np.float64)
    rp, rpi = O.to_ref_layout(phi), O.to_ref_layout(pi)
    out = {}
    for prec in (0, 1):
        with PL.Lattice(PL.Params(N=N, precision=prec)) as lat:
            lat.upload(rp, rpi)
            out[prec] = [lat.correlation_functions(), lat.spectrum_uniform(64), lat.spectrum_uniform(1024)]
            t, b = lat.spectrum_timing()
            assert t > 0 and b > 0
    for (F32, K32, Q32, C32), (F64, K64, Q64, C64) in zip(out[1], out[0]):
        assert np.array_equal(C32, C64) and C32.sum() == N ** 3
        np.testing.assert_allclose(F32, F64, rtol=1e-5, atol=1e-12 * np.abs(F64).max())
        np.testing.assert_allclose(K32, K64, rtol=1e-5, atol=1e-12 * np.abs(K64).max())
        np.testing.assert_allclose(Q32, Q64, rtol=0, atol=1e-5 * np.abs(Q64).max())
