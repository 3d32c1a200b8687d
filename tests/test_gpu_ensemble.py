"""Batched ensemble (phn_ensemble_*) against single-lattice runs.

A member of the ensemble must evolve exactly as a single-lattice handle with
the same inputs (same per-site arithmetic): fields bit-identical, island
counts identical, averages equal up to FP32 summation order (relative 1e-6,
extrema exact)."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SQ6 = 6 ** 0.5


def members():
    from phinum_gb300 import lattice as PL
    ms, fields = [], []
    spec = [(32, 0, 1.0, 0.1), (32, 1, -1.0, 0.0), (64, 0, 0.9, 0.15), (32, 0, 1.1, 0.05), (64, 1, -1.0, 0.0),
            (128, 0, 1.2, 0.2), (32, 0, 0.8, 0.12)]
    for i, (N, th, phi0, g) in enumerate(spec):
        if th == 0:
            p = PL.Params(N=N, precision=1, theory=0, kappa=(0.3 / g) ** 0.5)
        else:
            p = PL.Params(N=N, precision=1, theory=1, mass_mode=-1, lambda_mode=1, h=SQ6 * 0.05)
        phi, pi = inputs.lattice_fields(N, 1, 100 + i, phi0=SQ6 * phi0)
        ms.append(p)
        fields.append((O.to_ref_layout(phi), O.to_ref_layout(pi)))
    return ms, fields


@pytest.mark.parametrize("tile", [0, 1, 3, 6, 9, 10])  # scalar tiles, then x4 tiles with 8, 4, 2 warps
def test_members_match_single_lattice_runs(tile):
    from phinum_gb300 import lattice as PL
    ms, fields = members()
    steps = 137  # two 50-step graph chunks and a remainder
    with PL.Ensemble(ms) as ens:
        ens.set_tile(tile)
        for m, (phi, pi) in enumerate(fields):
            ens.upload(m, phi, pi)
        ens.evolve(steps)
        avg = ens.averages()
        for m, p in enumerate(ms):
            with PL.Lattice(p) as lat:
                lat.upload(*fields[m])
                lat.evolve(steps)
                sphi, spi = lat.download()
                savg = lat.volume_averages()
                ephi, epi = ens.download(m)
                N = p.N
                assert np.array_equal(ephi, sphi), m
                assert np.array_equal(epi[N * N:-N * N], spi[N * N:-N * N]), m
                assert np.array_equal(avg[m, 17:23], savg[17:23]), m
                np.testing.assert_allclose(avg[m, 9:17], savg[9:17], rtol=1e-6, atol=1e-9)
                thr = float(np.quantile(np.sqrt(sphi[N * N:-N * N] ** 2 + spi[N * N:-N * N] ** 2), 0.9))
                n_ens, _ = ens.islands(m, thr)
                lab, recs = lat.full_analysis(thr, labels=True)
                assert n_ens == recs.shape[0], m
                if m == 0:
                    olab, orecs = O.islands(O.Params(N=N), sphi, spi, thr)
                    assert np.array_equal(lab, olab) and orecs.shape[0] == n_ens


@pytest.mark.parametrize("tile", [0, 6])  # a scalar tile and an x4 tile
def test_expanding_members_match_single_lattice_runs(tile):
    """The expanding box (one H0, one clock): a member's fields equal a
    single expanding lattice's bit for bit (the kick's couplings scaled by
    the step's scale factor with the handle's expressions), the averages'
    extrema exactly and their sums to FP32 summation order, the time and
    scale-factor columns exactly; island counts equal."""
    from phinum_gb300 import lattice as PL
    ms, fields = members()
    ms, fields = ms[:3], fields[:3]
    for p in ms:
        p.expansion, p.H0, p.T0 = 1, 0.05, 2.0
    steps = 137
    with PL.Ensemble(ms) as ens:
        ens.set_tile(tile)
        for m, (phi, pi) in enumerate(fields):
            ens.upload(m, phi, pi)
        ens.evolve(steps)
        avg = ens.averages()
        for m, p in enumerate(ms):
            with PL.Lattice(p) as lat:
                lat.upload(*fields[m])
                lat.evolve(steps)
                sphi, spi = lat.download()
                savg = lat.volume_averages()
                ephi, epi = ens.download(m)
                N = p.N
                assert np.array_equal(ephi, sphi), m
                assert np.array_equal(epi[N * N:-N * N], spi[N * N:-N * N]), m
                assert avg[m, 0] == savg[0] and avg[m, 25] == savg[25] and savg[25] > 1.0, m
                assert np.array_equal(avg[m, 17:23], savg[17:23]), m
                np.testing.assert_allclose(avg[m, 9:17], savg[9:17], rtol=1e-6, atol=1e-9)
                thr = float(np.quantile(np.sqrt(sphi[N * N:-N * N] ** 2 + spi[N * N:-N * N] ** 2), 0.9))
                n_ens, _ = ens.islands(m, thr)
                _, recs = lat.full_analysis(thr, labels=False)
                assert n_ens == recs.shape[0], m


def test_autotune_keeps_state():
    from phinum_gb300 import lattice as PL
    ms, fields = members()
    with PL.Ensemble(ms) as ens:
        for m, (phi, pi) in enumerate(fields):
            ens.upload(m, phi, pi)
        ens.evolve(3)
        before = [ens.download(m) for m in range(len(ms))]
        t, ms_best = ens.autotune(3)
        assert t >= 0 and ms_best > 0
        after = [ens.download(m) for m in range(len(ms))]
        for (a0, b0), (a1, b1) in zip(before, after):
            assert np.array_equal(a0, a1) and np.array_equal(b0, b1)


def test_ensemble_validation():
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([PL.Params(N=32, precision=1), PL.Params(N=32, precision=0)])
    assert e.value.code == L.ERR_UNSUPPORTED
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([PL.Params(N=32, precision=1), PL.Params(N=32, precision=1, dt=0.05)])
    assert e.value.code == L.ERR_INVALID
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([PL.Params(N=48, precision=1)])
    assert e.value.code == L.ERR_UNSUPPORTED
    # one clock: every member expanding with one H0, or none
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([PL.Params(N=32, precision=1, expansion=1), PL.Params(N=32, precision=1)])
    assert e.value.code == L.ERR_INVALID
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([PL.Params(N=32, precision=1, expansion=1, H0=0.05),
                     PL.Params(N=32, precision=1, expansion=1, H0=0.06)])
    assert e.value.code == L.ERR_INVALID
