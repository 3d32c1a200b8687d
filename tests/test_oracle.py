"""Pins the CPU oracle (oracle/phinum_oracle.c) to the reference.

The fixtures in tests/golden/ were produced by the reference's own sources
(dynamics.cpp, fieldanalysis.cpp, momentumspace.cpp, islands.cpp compiled
unchanged against single-rank shims, oracle/build_ref.sh).  The oracle must
reproduce every FP64 field, SO row and island label bit for bit; spectra use
a different FFT, so their values agree to rounding and their bin counts
exactly.
"""
import os

import numpy as np
import pytest

import fixtures
from oracle import oracle as O

CASES = fixtures.names()
ROW_COLS = slice(0, 23)  # t .. max_abs_pos: everything the reference computes
SF_COL = 25               # the expanding box's scale factor


def params(d):
    return O.Params(a=d["a"], dt=d["dt"], **d["params"])


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(name):
    d = fixtures.load(name)
    p = params(d)
    phi_i, pi_i = fixtures.inputs_for(d)
    if "phi_init" in d:
        assert np.array_equal(phi_i, d["phi_init"]) and np.array_equal(pi_i, d["pi_init"])
    nthreads = min(8, O.max_threads(False) if hasattr(O, "max_threads") else 1)

    # SO rows over the whole run: bit-exact
    phi, pi = O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc)
    rows, clk = O.run_loop(p, phi, pi, d["steps"], d["tso"], nthreads=nthreads)
    assert rows.shape[0] == d["rows"].shape[0]
    assert np.array_equal(rows[:, ROW_COLS], d["rows"][:, ROW_COLS])
    if p.expansion:
        assert np.array_equal(rows[:, SF_COL], d["rows"][:, SF_COL]) and rows[-1, SF_COL] > 1.0

    # fields at each checkpoint: bit-exact
    phi, pi = O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc)
    clock = O.Clock(p)
    done = 0
    for c in fixtures.checkpoints(d):
        O.evolve(p, phi, pi, c - done, clock, nthreads=nthreads)
        done = c
        phi_c, pi_c = O.from_ref_layout(phi, p.N, p.Nc), O.from_ref_layout(pi, p.N, p.Nc)
        assert fixtures.digest(phi_c) == str(d[f"phi_sha_{c}"]), f"phi after {c} steps"
        assert fixtures.digest(pi_c) == str(d[f"pi_sha_{c}"]), f"pi after {c} steps"
        avg = O.averages(p, phi, pi, clock)
        assert np.array_equal(avg[ROW_COLS], d[f"avg_{c}"][ROW_COLS])
        if p.expansion:
            assert avg[SF_COL] == d[f"avg_{c}"][SF_COL]
    assert clock.tau == d["tau_end"] and clock.steps == d["steps_end"]

    # spectrum of the final state
    F, K, Q, C = O.spectrum(p, phi, pi)
    assert np.array_equal(C, d["spec_counts"])
    scale = np.abs(d["spec_F"]).max()
    np.testing.assert_allclose(F, d["spec_F"], rtol=1e-11, atol=1e-13 * scale)
    np.testing.assert_allclose(K, d["spec_K"], rtol=1e-11, atol=1e-13 * np.abs(d["spec_K"]).max())
    np.testing.assert_allclose(Q, d["spec_Q"], rtol=1e-9, atol=1e-12 * np.abs(d["spec_Q"]).max())

    # islands of the final state: labels and per-island statistics bit-exact
    if p.Nc == 1:
        labels, recs = O.islands(p, phi, pi, float(d["island_thres"]), clock=clock)
        lab = O.from_ref_layout(labels.astype(np.float64), p.N, 1)[0].astype(np.int32)
        assert fixtures.label_digest(lab) == str(d["island_labels_sha"])
        st = d["island_stats"]
        assert recs.shape[0] == st.shape[0]
        cols = [O.ISL[k] for k in ("index", "volume", "pot_en", "kin_en", "grad_en", "av_phi",
                                   "peak_pos", "peak_value")]
        assert np.array_equal(recs[:, cols], st)


def test_oracle_threads_do_not_change_results():
    d = fixtures.load("t0_n12")
    p = params(d)
    phi_i, pi_i = fixtures.inputs_for(d)
    outs = []
    for nt in (1, 3):
        phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
        O.evolve(p, phi, pi, 20, nthreads=nt)
        outs.append((phi, pi))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_spectrum_counts_cover_every_mode():
    for N in (8, 12, 32, 64):
        p = O.Params(N=N)
        nb, bs = O.spectrum_bins(p)
        phi = O.to_ref_layout(np.zeros((N, N, N)))
        F, K, Q, C = O.spectrum(p, phi, phi.copy())
        assert C.sum() == N ** 3  # every lattice mode lands in exactly one bin
        # int(sqrt(3)/sin(pi/N) + 0.5) + 2 (momentumspace.cpp:40-47)
        assert nb == {8: 7, 12: 9, 32: 20, 64: 37}[N]


@pytest.mark.skipif(not all(O.ref_available(t, "f64", e) for t in range(6) for e in (0, 1)),
                    reason="reference pin not built here (oracle/build_ref.sh)")
@pytest.mark.parametrize("theory,N,Nc,expansion", [(0, 6, 1, 0), (1, 10, 1, 0), (0, 8, 3, 0), (2, 6, 1, 0),
                                                   (3, 6, 1, 0), (4, 8, 1, 0), (5, 6, 1, 0), (0, 6, 2, 1),
                                                   (1, 8, 1, 1), (2, 6, 1, 1), (3, 6, 1, 1), (4, 6, 1, 1),
                                                   (5, 6, 1, 1), (1, 6, 4, 0), (1, 6, 3, 1), (0, 6, 4, 1)])
def test_oracle_matches_reference_live(theory, N, Nc, expansion, tmp_path):
    """Runs the reference pin in a child process on fresh random inputs."""
    import subprocess
    import sys
    import textwrap
    import os
    code = textwrap.dedent(f"""
        import sys, numpy as np
        sys.path.insert(0, {os.getcwd()!r}); sys.path.insert(0, {os.path.dirname(O.HERE)!r})
        from oracle import oracle as O
        kw = {{0: dict(theory=0, mass_mode=1, lambda_mode=-1, kappa=3**0.5),
              1: dict(theory=1, mass_mode=-1, lambda_mode=1, h=0.3),
              2: dict(theory=2, m_sqr=0.49), 3: dict(theory=3, m_sqr=9.0, m_mono_sqr=1.0),
              4: dict(theory=4, mass_mode=1, lambda_mode=1, g=2.0), 5: dict(theory=5, p_mono=-0.5)}}[{theory}]
        p = O.Params(N={N}, Nc={Nc}, expansion={expansion}, H0=0.05, T0=0.5 * {expansion}, **kw)
        rng = np.random.default_rng({N})
        phi = O.to_ref_layout(2.0 + 0.5 * rng.standard_normal(({Nc}, {N}, {N}, {N})), {Nc})
        pi = O.to_ref_layout(0.5 * rng.standard_normal(({Nc}, {N}, {N}, {N})), {Nc})
        R = O.Reference(p); R.set_fields(phi, pi)
        rr = R.run_loop(37, 0.1)
        rf = R.get_fields()
        rows, clk = O.run_loop(p, phi, pi, 37, 0.1)
        assert np.array_equal(rr[:, :23], rows[:, :23])
        assert np.array_equal(rf[0], phi) and np.array_equal(rf[1], pi)
        assert R.expansion_state() == (clk.tau_c, clk.sf)
        if {expansion}:
            assert np.array_equal(rr[:, 25], rows[:, 25])
        if {Nc} == 1:
            thr = float(np.quantile(np.sqrt(phi**2 + pi**2), 0.9))
            l1, s1 = R.islands(thr); l2, s2 = O.islands(p, phi, pi, thr, clock=clk)
            assert np.array_equal(l1, l2)
            cols = [O.ISL[k] for k in ("index", "volume", "pot_en", "kin_en", "grad_en", "av_phi", "peak_pos",
                                       "peak_value")]
            assert np.array_equal(s1, s2[:, cols])
        print("ok")
    """)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr


F32_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "f32")


@pytest.mark.parametrize("name", sorted(f[:-4] for f in os.listdir(F32_DIR)))
def test_single_precision_port_matches_reference_float_build(name):
    """orc_evolve_f32, the restatement of the reference's doubleprecision -1
    build (float fields and clock, double literals), against that build's own
    output (fixtures from oracle/_ref/libphinum_ref_t{0,1}_f32.so): float
    fields bit-identical after 100 steps, and the float clock."""
    import json
    import inputs
    with np.load(os.path.join(F32_DIR, name + ".npz")) as z:
        d = {k: z[k] for k in z.files}
    pd = json.loads(str(d["params"]))
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, int(d["seed"]), phi0=float(d["phi0"]))
    phi = O.to_ref_layout(phi_i, p.Nc).astype(np.float32)
    pi = O.to_ref_layout(pi_i, p.Nc).astype(np.float32)
    clock = O.evolve_f32(p, phi, pi, int(d["steps"]))
    slab = p.Nc * p.N * p.N
    assert np.array_equal(phi, d["phi"])
    assert np.array_equal(pi[slab:-slab], d["pi"][slab:-slab])
    assert clock.tau == float(d["tau"]) and clock.steps == int(d["steps"])
    # the timing build (-O3 -ffast-math, the reference's flags) on all threads runs the same steps
    phi2 = O.to_ref_layout(phi_i, p.Nc).astype(np.float32)
    pi2 = O.to_ref_layout(pi_i, p.Nc).astype(np.float32)
    O.evolve_f32(p, phi2, pi2, int(d["steps"]), nthreads=O.max_threads(True), fast=True)
    np.testing.assert_allclose(phi2, phi, rtol=0, atol=1e-4)


EPS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eps")
EPS = sorted(n[:-4] for n in os.listdir(EPS_DIR) if n.endswith(".npz")) if os.path.isdir(EPS_DIR) else []


@pytest.mark.parametrize("name", EPS)
def test_energy_density_analysis_matches_reference_fixture(name):
    """withEnergyPS 1 with EnergybasedID 1, the reference builds that compile
    it (theories 2-5, static and expanding): Delta bit-exact, the threshold
    4 <rho> that Full_Analysis sets, the Delta mask's labels and records (peak
    and Peak_value by Delta) bit-exact, the density-contrast spectrum within
    the rounding of the two FFTs."""
    import json
    import inputs
    d = np.load(os.path.join(EPS_DIR, name + ".npz"))
    pd = json.loads(str(d["params"]))
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, int(d["seed"]), phi0=float(d["phi0"]))
    phi, pi = O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc)
    clock = O.Clock(p)
    O.evolve(p, phi, pi, int(d["steps"]), clock)
    slab = p.Nc * p.N * p.N
    assert np.array_equal(phi[slab:-slab], d["phi"][slab:-slab]) and np.array_equal(pi[slab:-slab], d["pi"][slab:-slab])
    delta = O.delta(p, phi, pi, clock)
    assert np.array_equal(delta, d["delta"])
    thr = 4.0 * O.averages(p, phi, pi, clock)[O.AVG["energy"]]
    assert thr == float(d["thres"])
    labels, recs = O.islands(p, phi, pi, thr, mode=2, clock=clock)
    assert np.array_equal(labels, d["labels"])
    st = d["stats"]
    assert recs.shape[0] == st.shape[0] > 0
    cols = [O.ISL[k] for k in ("index", "volume", "pot_en", "kin_en", "grad_en", "av_phi", "peak_pos", "peak_value")]
    assert np.array_equal(recs[:, cols], st)
    D, C = O.spectrum_energy(p, phi, pi, clock)
    assert np.array_equal(C, d["counts"])
    np.testing.assert_allclose(D, d["D"], rtol=1e-10, atol=1e-12 * np.abs(d["D"]).max())


def test_energy_density_analysis_is_refused_where_the_reference_does_not_compile_it():
    p = O.Params(N=8, theory=0)
    phi = O.to_ref_layout(np.ones((8, 8, 8)))
    with pytest.raises(ValueError):
        O.delta(p, phi, phi.copy())
    with pytest.raises(ValueError):
        O.islands(p, phi, phi.copy(), 1.0, mode=2)
