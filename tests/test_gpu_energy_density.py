"""GPU energy-density analysis (the reference's withEnergyPS 1 with
EnergybasedID 1) against fixtures from the reference builds that compile it
(tests/golden/eps: theories 2-5, static and expanding box) and against the
oracle.

Tolerances:
  FP64 fields (the reference's own, uploaded after the same number of steps
  sets the clock): island labels, sizes and peak positions exact; the threshold
  4 <rho>, the island energies and Peak_value (Delta at the peak) within
  1e-11 relative (theories 2, 3 and 5 evaluate cos and pow with CUDA's
  functions, so FP64 agrees to rounding, not bitwise); the density-contrast
  spectrum within 1e-9 relative (cuFFT against the reference's transform).
  FP32 fields: the contrast spectrum within 1e-4 relative of the oracle's
  FP64 spectrum of the same (FP32-valued) fields; island counts within 2 of
  the oracle's (a site within FP32 rounding of the threshold may fall on
  either side).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eps")
EPS = sorted(n[:-4] for n in os.listdir(EPS_DIR) if n.endswith(".npz"))


def load(name):
    d = np.load(os.path.join(EPS_DIR, name + ".npz"))
    return d, json.loads(str(d["params"]))


def lattice(pd, precision, seed, phi0, steps):
    """A lattice of params pd with the fixture's inputs evolved `steps` steps
    on the GPU (FP64: the reference's fields bit for bit for theory 4, to
    rounding for the sin/cos/pow theories)."""
    import inputs
    from phinum_gb300 import lattice as PL
    p = PL.Params(precision=precision, a=0.25, dt=0.08, T0=0.0, **pd)
    lat = PL.Lattice(p)
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=phi0)
    lat.upload(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    lat.evolve(steps)
    return lat


@pytest.mark.parametrize("name", EPS)
def test_delta_islands_and_contrast_spectrum_match_reference(name):
    d, pd = load(name)
    lat = lattice(pd, 0, int(d["seed"]), float(d["phi0"]), int(d["steps"]))
    N = pd["N"]
    slab = N * N
    phi, pi = lat.download()
    # the evolution: bit-exact for theory 4, to rounding for 2, 3, 5 (CUDA's
    # sin, cos and pow); the analysis then starts from the reference's own
    # fields (the clock stays where the steps left it)
    for got, want in ((phi, d["phi"]), (pi, d["pi"])):
        if pd["theory"] == 4:
            assert np.array_equal(got[slab:-slab], want[slab:-slab])
        else:
            np.testing.assert_allclose(got[slab:-slab], want[slab:-slab], rtol=0, atol=1e-12)
    lat.upload(d["phi"], d["pi"])
    # Full_Analysis' threshold, 4 <rho> (islands.cpp:783-786)
    thr = 4.0 * lat.volume_averages()[O.AVG["energy"]]
    np.testing.assert_allclose(thr, float(d["thres"]), rtol=1e-11)
    lab, recs = lat.full_analysis(float(d["thres"]), mode=2)
    assert np.array_equal(lab, d["labels"])
    st = d["stats"]  # index, V, PotEn, KinEn, GradEn, avPhi, peak pos, Peak_value
    I = {k: i for i, k in enumerate(O.ISLAND_FIELDS)}
    assert recs.shape[0] == st.shape[0] > 0
    assert np.array_equal(recs[:, I["index"]], st[:, 0]) and np.array_equal(recs[:, I["volume"]], st[:, 1])
    assert np.array_equal(recs[:, I["peak_pos"]], st[:, 6])
    for j, k in ((2, "pot_en"), (3, "kin_en"), (4, "grad_en"), (5, "av_phi"), (7, "peak_value")):
        np.testing.assert_allclose(recs[:, I[k]], st[:, j], rtol=1e-11, atol=1e-13 * np.abs(st[:, j]).max())
    D, C = lat.spectrum_energy()
    assert np.array_equal(C, d["counts"])
    np.testing.assert_allclose(D, d["D"], rtol=1e-9, atol=1e-12 * np.abs(d["D"]).max())
    lat.close()


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("name", ["eps_t3_n12", "eps_t5_n12"])
def test_fp32_delta_analysis_tracks_the_oracle(name, precision):
    d, pd = load(name)
    lat = lattice(pd, precision, int(d["seed"]), float(d["phi0"]), int(d["steps"]))
    phi, pi = lat.download()
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    thr = float(d["thres"])
    lab, recs = lat.full_analysis(thr, mode=2)
    olab, orecs = O.islands(p, phi, pi, thr, mode=2)
    assert abs(recs.shape[0] - orecs.shape[0]) <= 2
    D, C = lat.spectrum_energy()
    oD, oC = O.spectrum_energy(p, phi, pi)
    assert np.array_equal(C, oC)
    np.testing.assert_allclose(D, oD, rtol=1e-4, atol=1e-6 * np.abs(oD).max())
    lat.close()


def test_delta_at_larger_sizes_matches_the_oracle():
    """64^3 and a 48^3 lattice (the untiled labelling, edges that are not
    multiples of 32): Delta-mask labels and sizes equal the oracle's BFS on the
    same FP64 fields, z open and periodic."""
    import inputs
    from phinum_gb300 import lattice as PL
    for N in (64, 48):
        pd = dict(N=N, Nc=1, theory=3, mass_mode=1, lambda_mode=1, m_sqr=9.0, kappa=1.0, h=0.0, m_mono_sqr=1.0)
        p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
        phi_i, pi_i = inputs.lattice_fields(N, 1, 81, phi0=0.0)
        phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
        thr = 4.0 * O.averages(p, phi, pi)[O.AVG["energy"]]
        lat = PL.Lattice(PL.Params(precision=0, a=0.25, dt=0.08, T0=0.0, **pd))
        lat.upload(phi, pi)
        for zper in (0, 1):
            lab, recs = lat.full_analysis(thr, mode=2, z_periodic=bool(zper))
            olab, orecs = O.islands(p, phi, pi, thr, mode=2, zper=zper)
            assert np.array_equal(lab, olab), (N, zper)
            assert np.array_equal(recs[:, 1], orecs[:, 1])
            I = {k: i for i, k in enumerate(O.ISLAND_FIELDS)}
            assert np.array_equal(recs[:, I["peak_pos"]], orecs[:, I["peak_pos"]])
            np.testing.assert_allclose(recs[:, I["peak_value"]], orecs[:, I["peak_value"]], rtol=1e-12)
        lat.close()


def test_energy_density_analysis_is_refused_for_theories_0_and_1():
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL
    lat = PL.Lattice(PL.Params(N=16, theory=0))
    with pytest.raises(L.PhnError) as e:
        lat.full_analysis(1.0, mode=2)
    assert e.value.code == L.ERR_UNSUPPORTED
    with pytest.raises(L.PhnError) as e:
        lat.spectrum_energy()
    assert e.value.code == L.ERR_UNSUPPORTED
    lat.close()
