"""Config-mode spectrum on the GPU (phn_spectrum_uniform) against the
oracle: counts exact; FP64 sums to 1e-10 of the largest bin, FP32 to 1e-4
relative (1e-5 of the largest bin absolute)."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,nbins,precision", [(16, 64, 0), (32, 64, 0), (32, 64, 1), (64, 64, 1), (32, 7, 0)])
def test_uniform_spectrum_matches_oracle(N, nbins, precision):
    from phinum_gb300 import lattice as PL
    phi, pi = inputs.lattice_fields(N, 1, seed=40 + N)
    rp, rpi = O.to_ref_layout(phi), O.to_ref_layout(pi)
    oF, oK, oQ, oC = O.spectrum_uniform(O.Params(N=N), rp, rpi, nbins)
    with PL.Lattice(PL.Params(N=N, precision=precision)) as lat:
        lat.upload(rp, rpi)
        F, K, Q, C = lat.spectrum_uniform(nbins)
        # the reference-mode spectrum on the same handle is unaffected
        rF, _, _, rC = lat.correlation_functions()
    assert np.array_equal(C, oC)
    assert C.sum() == N ** 3 and rC.sum() == N ** 3
    rtol, atol = (1e-10, 1e-10) if precision == 0 else (1e-4, 1e-5)
    for got, ref in ((F, oF), (K, oK), (Q, oQ)):
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=atol * np.abs(ref).max())
    assert abs(F.sum() - rF.sum()) <= (1e-10 if precision == 0 else 1e-5) * rF.sum()


def test_uniform_spectrum_rejects_bad_bin_counts():
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    with PL.Lattice(PL.Params(N=16)) as lat:
        for nb in (0, -3, 1025):
            assert lat.lib.phn_spectrum_uniform(lat.h, nb, None, None, None, None) == L.ERR_INVALID
        F, K, Q, C = lat.spectrum_uniform(1024)  # the largest bin count
        assert C.sum() == 16 ** 3
