"""Config-mode spectrum (uniform |p| bins on [0, p_max]) in the oracle,
checked against an independent numpy restatement: the full-grid FFT with
every mode counted once (conjugate symmetry makes that equal to the
reference's half-space walk with doubled interior py planes)."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O


def numpy_uniform(phi, pi, N, a, nbins):
    """phi, pi as [z][y][x] arrays (one component)."""
    n = np.arange(N)
    p1 = np.where(n < N // 2 + 1, 2.0 / a * np.sin(n * np.arccos(-1.0) / N),
                  -2.0 / a * np.sin(n * np.arccos(-1.0) / N))
    pz, py, px = np.meshgrid(p1, p1, p1, indexing="ij")
    psqr = (px * px + py * py) + pz * pz
    width = np.sqrt(3.0 * (4.0 / (a * a))) / nbins
    b = np.minimum((np.sqrt(psqr) / width).astype(np.int64), nbins - 1).ravel()
    f3 = a * a * a
    Fp, Pp = np.fft.fftn(phi) * f3, np.fft.fftn(pi) * f3
    F = np.bincount(b, (np.abs(Fp) ** 2).ravel(), nbins)
    K = np.bincount(b, (np.abs(Pp) ** 2).ravel(), nbins)
    Q = np.bincount(b, (Fp.real * Pp.real + Fp.imag * Pp.imag).ravel(), nbins)
    C = np.bincount(b, minlength=nbins)
    return F, K, Q, C


@pytest.mark.parametrize("N,nbins", [(8, 64), (12, 17), (16, 64)])
def test_oracle_uniform_matches_numpy(N, nbins):
    p = O.Params(N=N)
    phi, pi = inputs.lattice_fields(N, 1, seed=N + nbins)
    F, K, Q, C = O.spectrum_uniform(p, O.to_ref_layout(phi), O.to_ref_layout(pi), nbins)
    nF, nK, nQ, nC = numpy_uniform(phi, pi, N, p.a, nbins)
    assert np.array_equal(C, nC)
    assert C.sum() == N ** 3
    for got, ref in ((F, nF), (K, nK), (Q, nQ)):
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_uniform_and_reference_bins_hold_the_same_total():
    N = 16
    p = O.Params(N=N)
    phi, pi = inputs.lattice_fields(N, 1, seed=3)
    rp, rpi = O.to_ref_layout(phi), O.to_ref_layout(pi)
    F, K, Q, C = O.spectrum_uniform(p, rp, rpi, 64)
    rF, rK, rQ, rC = O.spectrum(p, rp, rpi)
    assert C.sum() == rC.sum() == N ** 3
    for u, r in ((F, rF), (K, rK), (Q, rQ)):
        assert abs(u.sum() - r.sum()) <= 1e-11 * np.abs(r).sum()
