"""GPU parity: the CUDA path through the C ABI against the reference's own
outputs (tests/golden/, produced by the reference sources) and the oracle.

Tolerances
  FP64 fields and SO-row extrema: bit-exact (same IEEE operations in the
      reference's order) for theories 0, 1 and 4; theories 2, 3 and 5 call
      sin/cos/pow, whose CUDA results may differ from the C library's in the
      last bit: fields and extrema within 1e-12 of the largest value after
      100 steps, extrema positions exact.
  FP64 sums (averages, energies): relative 1e-11 -- tree order vs the
      reference's sequential sums.
  FP64 spectra: relative 1e-10 of the largest bin (cuFFT vs the oracle FFT);
      bin counts exact.
  FP32 fields after 100 steps: absolute 2e-4 (fields are O(1)); averages
      relative 2e-5.  Compensated FP32: absolute 2e-5.
  Islands: labels, counts and sizes exact; island sums relative 1e-11.
"""
import ctypes
import os

import numpy as np
import pytest

import fixtures
from rows import assert_fp32_sums_close
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROW_COLS = slice(0, 23)
SUM_COLS = [1, 5, 9, 10, 11, 12, 13, 14, 15, 16]      # phi0, pi0, phi2 .. charge
EXACT_COLS = [0, 17, 18, 19, 20, 21, 22]               # t, extrema values and positions
TRANSCENDENTAL = {2, 3, 5}                             # theories whose force calls sin / pow


def fp64_exact(d) -> bool:
    return d["params"]["theory"] not in TRANSCENDENTAL


def gpu():
    from phinum_gb300 import lattice as PL
    return PL


def gparams(d, precision):
    PL = gpu()
    return PL.Params(precision=precision, a=d["a"], dt=d["dt"], **d["params"])


def start(d, precision):
    PL = gpu()
    p = gparams(d, precision)
    lat = PL.Lattice(p)
    phi_i, pi_i = fixtures.inputs_for(d)
    lat.upload(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    return lat, p


def interior(flat, p):
    return O.from_ref_layout(flat, p.N, p.Nc)


CASES = fixtures.names()


@pytest.mark.parametrize("name", CASES)
def test_fp64_fields_bit_exact(name):
    d = fixtures.load(name)
    lat, p = start(d, 0)
    done = 0
    for c in fixtures.checkpoints(d):
        lat.evolve(c - done)
        done = c
        phi, pi = lat.download()
        a = lat.volume_averages()
        ref = d[f"avg_{c}"]
        if fp64_exact(d):
            assert fixtures.digest(interior(phi, p)) == str(d[f"phi_sha_{c}"]), f"phi after {c}"
            assert fixtures.digest(interior(pi, p)) == str(d[f"pi_sha_{c}"]), f"pi after {c}"
            assert np.array_equal(a[EXACT_COLS[1:]], ref[EXACT_COLS[1:]])
        else:
            for got, want in ((interior(phi, p), d[f"phi_{c}"]), (interior(pi, p), d[f"pi_{c}"])):
                assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), f"after {c}"
            assert np.array_equal(a[[20, 21, 22]], ref[[20, 21, 22]])
            np.testing.assert_allclose(a[[17, 18, 19]], ref[[17, 18, 19]], rtol=1e-12)
        np.testing.assert_allclose(a[SUM_COLS], ref[SUM_COLS], rtol=1e-11, atol=1e-14)
    t, s = lat.time()
    assert t == d["tau_end"] and s == d["steps_end"]
    lat.close()


@pytest.mark.parametrize("name", CASES)
def test_fp64_run_loop_rows(name):
    d = fixtures.load(name)
    lat, p = start(d, 0)
    rows = lat.run_loop(d["steps"], d["tso"])
    ref = d["rows"]
    assert rows.shape[0] == ref.shape[0]
    if fp64_exact(d):
        assert np.array_equal(rows[:, EXACT_COLS], ref[:, EXACT_COLS])
    else:
        assert np.array_equal(rows[:, [0, 20, 21, 22]], ref[:, [0, 20, 21, 22]])
        np.testing.assert_allclose(rows[:, [17, 18, 19]], ref[:, [17, 18, 19]], rtol=1e-12)
    np.testing.assert_allclose(rows[:, SUM_COLS], ref[:, SUM_COLS], rtol=1e-11, atol=1e-14)
    # the fused rows leave the fields exactly where plain evolve() does
    phi, pi = lat.download()
    c = max(fixtures.checkpoints(d))
    if c == d["steps"] and fp64_exact(d):
        assert fixtures.digest(interior(phi, p)) == str(d[f"phi_sha_{c}"])
    lat.close()


@pytest.mark.parametrize("precision,atol", [(1, 2e-4), (2, 2e-5)])
@pytest.mark.parametrize("name", ["t0_n8", "t1_n8", "t0_n12", "t0_n16_nc2", "t0_n8_nc3", "t1_n12_nc4", "t2_n8", "t3_n8",
                                  "t4_n8", "t5_n8", "t2_n8_nc2", "t3_n8_nc3", "t4_n8_nc2", "t5_n8_nc4"])
def test_fp32_fields_close(name, precision, atol):
    d = fixtures.load(name)
    lat, p = start(d, precision)
    last = max(fixtures.checkpoints(d))
    lat.evolve(last)
    phi, pi = lat.download()
    np.testing.assert_allclose(interior(phi, p), d[f"phi_{last}"], rtol=0, atol=atol)
    np.testing.assert_allclose(interior(pi, p), d[f"pi_{last}"], rtol=0, atol=atol)
    rows = lat.run_loop(0, 1.0)  # nothing due: no rows
    assert rows.shape[0] == 0
    lat.close()


@pytest.mark.parametrize("precision,rtol", [(1, 2e-5), (2, 2e-6)])
@pytest.mark.parametrize("name", ["c0_n64", "t1_n32"])
def test_fp32_rows_close(name, precision, rtol):
    d = fixtures.load(name)
    lat, p = start(d, precision)
    steps = min(d["steps"], 500)
    rows = lat.run_loop(steps, d["tso"])
    ref = d["rows"][: rows.shape[0]]
    assert rows.shape[0] == ref.shape[0]
    assert np.array_equal(rows[:, 0], ref[:, 0])  # stamps come from the same FP64 clock
    for col in ("energy", "interaction", "phi2", "pi2", "phi4"):
        j = O.AVG[col]
        np.testing.assert_allclose(rows[:, j], ref[:, j], rtol=rtol, atol=rtol * np.abs(ref[:, j]).max())
    lat.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_spectrum(name, precision):
    d = fixtures.load(name)
    lat, p = start(d, precision)
    lat.evolve(d["steps"]) if precision == 0 else None
    F, K, Q, C = lat.correlation_functions()
    assert np.array_equal(C, d["spec_counts"])
    if precision == 0:
        for got, key in ((F, "spec_F"), (K, "spec_K"), (Q, "spec_Q")):
            ref = d[key]
            np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
    else:
        # FP32 spectrum of the initial fields against the oracle's FP64 spectrum
        phi_i, pi_i = fixtures.inputs_for(d)
        op = O.Params(a=d["a"], dt=d["dt"], **d["params"])
        oF, oK, oQ, oC = O.spectrum(op, O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
        assert np.array_equal(C, oC)
        for got, ref in ((F, oF), (K, oK), (Q, oQ)):
            np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-5 * np.abs(ref).max())
    lat.close()


@pytest.mark.parametrize("name", [n for n in CASES if fixtures.load(n)["params"]["Nc"] == 1])
def test_islands_fp64(name):
    d = fixtures.load(name)
    lat, p = start(d, 0)
    lat.evolve(d["steps"])
    lab, recs = lat.full_analysis(float(d["island_thres"]))
    li = O.from_ref_layout(lab.astype(np.float64), p.N, 1)[0].astype(np.int32)
    assert fixtures.label_digest(li) == str(d["island_labels_sha"])
    st = d["island_stats"]  # index, V, PotEn, KinEn, GradEn, avPhi, peak pos, Peak_value
    assert recs.shape[0] == st.shape[0]
    I = {k: i for i, k in enumerate(O.ISLAND_FIELDS)}
    assert np.array_equal(recs[:, I["index"]], st[:, 0])
    assert np.array_equal(recs[:, I["volume"]], st[:, 1])
    for j, k in ((2, "pot_en"), (3, "kin_en"), (4, "grad_en"), (5, "av_phi")):
        np.testing.assert_allclose(recs[:, I[k]], st[:, j], rtol=1e-11, atol=1e-13)
    # peak: the reference keeps the first maximum of phi^2 in BFS order, this
    # implementation the smallest index among maxima -- equal unless tied
    if fp64_exact(d):
        assert np.array_equal(np.abs(recs[:, I["peak_value"]]), np.abs(st[:, 7]))
    else:
        np.testing.assert_allclose(np.abs(recs[:, I["peak_value"]]), np.abs(st[:, 7]), rtol=1e-12)
    lat.close()


def test_islands_energy_mask_and_z_periodic_match_oracle():
    d = fixtures.load("t1_n32")
    lat, p = start(d, 0)
    phi_i, pi_i = fixtures.inputs_for(d)
    op = O.Params(a=d["a"], dt=d["dt"], **d["params"])
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    rho_mean = O.averages(op, phi, pi)[O.AVG["energy"]]
    for mode, thr in ((0, 2.6), (1, 2.0 * rho_mean)):
        for zper in (0, 1):
            lab, recs = lat.full_analysis(thr, mode=mode, z_periodic=bool(zper))
            olab, orecs = O.islands(op, phi, pi, thr, mode=mode, zper=zper)
            assert np.array_equal(lab, olab), (mode, zper)
            assert recs.shape[0] == orecs.shape[0]
            assert np.array_equal(recs[:, 1], orecs[:, 1])  # sizes
            assert np.array_equal(recs[:, 9], orecs[:, 9])  # seeds
    lat.close()


def test_download_fills_ghost_slabs_like_exchange():
    d = fixtures.load("t0_n16_nc2")
    lat, p = start(d, 0)
    lat.evolve(3)
    phi, _ = lat.download()
    slab = p.Nc * p.N * p.N
    assert np.array_equal(phi[:slab], phi[p.N * slab:(p.N + 1) * slab])
    assert np.array_equal(phi[(p.N + 1) * slab:], phi[slab:2 * slab])
    # Pi's ghost slabs belong to the caller: exchange() never writes them
    from phinum_gb300 import _lib as L
    pi = np.full(p.field_len, 7.5)
    L.check(lat.lib.phn_download(lat.h, None, pi.ctypes.data_as(L._PD)))
    assert np.all(pi[:slab] == 7.5) and np.all(pi[-slab:] == 7.5)
    assert not np.any(pi[slab:-slab] == 7.5)
    lat.close()


def test_results_are_deterministic():
    d = fixtures.load("c0_n64")
    outs = []
    for _ in range(2):
        lat, p = start(d, 1)
        rows = lat.run_loop(120, d["tso"])
        F, K, Q, C = lat.correlation_functions()
        lab, recs = lat.full_analysis(2.6)
        outs.append((rows, F, K, Q, lab, recs[:, :2]))
        lat.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


def test_errors_are_status_codes():
    PL = gpu()
    from phinum_gb300 import _lib as L
    with pytest.raises(L.PhnError) as e:
        PL.Lattice(PL.Params(N=8, Nc=9))
    assert e.value.code == L.ERR_UNSUPPORTED
    with pytest.raises(L.PhnError) as e:
        PL.Lattice(PL.Params(N=8, theory=6))
    assert e.value.code == L.ERR_INVALID
    with pytest.raises(L.PhnError) as e:
        PL.Lattice(PL.Params(N=8, a=-1.0))
    assert e.value.code == L.ERR_INVALID
    lat = PL.Lattice(PL.Params(N=8, Nc=2))
    with pytest.raises(L.PhnError) as e:
        lat.full_analysis(1.0)
    assert e.value.code == L.ERR_UNSUPPORTED
    lat.close()
    # a NaN injected on the host is reported, not trapped
    lat = PL.Lattice(PL.Params(N=8))
    phi = O.to_ref_layout(np.ones((8, 8, 8)))
    phi[8 * 8 + 5] = np.nan
    lat.upload(phi, np.zeros_like(phi))
    with pytest.raises(L.PhnError) as e:
        lat.volume_averages()
    assert e.value.code == L.ERR_NONFINITE
    a = lat.volume_averages(allow_nonfinite=True)
    assert a[24] == 1.0
    lat.close()


@pytest.mark.parametrize("N", [128, 256])
def test_large_lattice_fp32_against_fp64(N):
    """Full-size properties: FP32 tracks the bit-exact FP64 path, mode counts
    cover every lattice mode, island partitions agree between precisions'
    shared inputs and the oracle."""
    import inputs
    PL = gpu()
    phi_i, pi_i = inputs.lattice_fields(N, 1, 11)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    res = {}
    for prec in (0, 1, 2):
        lat = PL.Lattice(PL.Params(N=N, precision=prec))
        lat.upload(phi, pi)
        rows = lat.run_loop(100, 1.0)
        F, K, Q, C = lat.correlation_functions()
        assert C.sum() == N ** 3
        res[prec] = (rows, lat.download()[0])
        lat.close()
    e64 = res[0][0][:, O.AVG["energy"]]
    for prec, tol in ((1, 1e-5), (2, 1e-6)):
        np.testing.assert_allclose(res[prec][0][:, O.AVG["energy"]], e64, rtol=tol)
        assert np.abs(res[prec][1] - res[0][1]).max() < 100 * tol
    # islands at full size: GPU labels = oracle BFS labels (FP64 inputs)
    lat = PL.Lattice(PL.Params(N=N, precision=0))
    lat.upload(phi, pi)
    thr = float(np.quantile(np.sqrt(phi_i ** 2 + pi_i ** 2), 0.9))
    lab, recs = lat.full_analysis(thr)
    op = O.Params(N=N)
    olab, orecs = O.islands(op, phi, pi, thr)
    assert np.array_equal(lab, olab)
    assert np.array_equal(recs[:, 1], orecs[:, 1])
    lat.close()


@pytest.mark.parametrize("theory", [0, 1])
@pytest.mark.parametrize("N", [128, 256, 384])
def test_tma_path_matches_plain_path_bit_for_bit(N, theory):
    """The TMA-pipelined FP32 step and the register z-marching step compute
    identical fields; their fused SO rows agree to FP32-summation rounding,
    extrema exactly."""
    import inputs
    PL = gpu()
    from phinum_gb300 import _lib as L
    phi_i, pi_i = inputs.lattice_fields(N, 1, 40 + theory, phi0=(-1) ** theory * 6 ** 0.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    kw = dict(theory=0) if theory == 0 else dict(theory=1, mass_mode=-1, lambda_mode=1, h=0.12247)
    import ctypes
    out = {}
    lat = PL.Lattice(PL.Params(N=N, precision=1, **kw))
    nv = ctypes.c_int()
    L.check(lat.lib.phn_num_variants(lat.h, ctypes.byref(nv)))
    lat.close()
    assert nv.value >= 2
    for path, variant in [(L.PATH_PLAIN, None)] + [(L.PATH_TMA, v) for v in range(nv.value)]:
        lat = PL.Lattice(PL.Params(N=N, precision=1, **kw))
        L.check(lat.lib.phn_set_path(lat.h, path))
        if variant is not None:
            L.check(lat.lib.phn_set_variant(lat.h, variant))
        lat.upload(phi, pi)
        rows = lat.run_loop(120, 0.5)
        lat.evolve(7)
        out[(path, variant)] = (rows,) + lat.download()
        lat.close()
    r0, f0, p0 = out[(L.PATH_PLAIN, None)]
    for key, (r1, f1, p1) in out.items():
        assert np.array_equal(f0, f1) and np.array_equal(p0[N * N:-N * N], p1[N * N:-N * N]), key
        assert np.array_equal(r0[:, 17:23], r1[:, 17:23]), key
        assert_fp32_sums_close(r1, r0)


def test_autotune_keeps_state_and_picks_a_variant():
    import ctypes
    import inputs
    PL = gpu()
    from phinum_gb300 import _lib as L
    N = 256
    phi_i, pi_i = inputs.lattice_fields(N, 1, 5)
    lat = PL.Lattice(PL.Params(N=N, precision=1))
    lat.upload(O.to_ref_layout(phi_i), O.to_ref_layout(pi_i))
    lat.evolve(3)
    before = lat.download()
    v, ms = ctypes.c_int(), ctypes.c_double()
    L.check(lat.lib.phn_autotune(lat.h, 5, ctypes.byref(v), ctypes.byref(ms)))
    after = lat.download()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert v.value >= -1 and ms.value > 0  # -1: the plain kernel was fastest
    lat.close()


@pytest.mark.parametrize("theory", [0, 1])
@pytest.mark.parametrize("N", [32, 64, 96])
def test_x4_path_matches_plain_path_bit_for_bit(N, theory):
    """The four-sites-per-thread FP32 step (every variant) against the register
    z-marching step at sizes without the TMA kernel: identical fields, SO rows
    to FP32-summation rounding, extrema exact."""
    import ctypes
    import inputs
    PL = gpu()
    from phinum_gb300 import _lib as L
    phi_i, pi_i = inputs.lattice_fields(N, 1, 60 + theory, phi0=(-1) ** theory * 6 ** 0.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    kw = dict(theory=0) if theory == 0 else dict(theory=1, mass_mode=-1, lambda_mode=1, h=0.12247)
    lat = PL.Lattice(PL.Params(N=N, precision=1, **kw))
    nv = ctypes.c_int()
    L.check(lat.lib.phn_num_variants(lat.h, ctypes.byref(nv)))
    lat.close()
    assert nv.value >= 2
    out = {}
    for variant in [None] + list(range(nv.value)):
        lat = PL.Lattice(PL.Params(N=N, precision=1, **kw))
        if variant is None:
            L.check(lat.lib.phn_set_path(lat.h, L.PATH_PLAIN))
        else:
            L.check(lat.lib.phn_set_variant(lat.h, variant))
            path = ctypes.c_int()
            L.check(lat.lib.phn_get_path(lat.h, ctypes.byref(path)))
            assert path.value == L.PATH_X4
        lat.upload(phi, pi)
        rows = lat.run_loop(120, 0.5)
        lat.evolve(7)
        avg = lat.volume_averages()
        out[variant] = (rows, avg) + lat.download()
        lat.close()
    r0, a0, f0, p0 = out[None]
    for key, (r1, a1, f1, p1) in out.items():
        assert np.array_equal(f0, f1) and np.array_equal(p0[N * N:-N * N], p1[N * N:-N * N]), key
        assert np.array_equal(r0[:, 17:23], r1[:, 17:23]), key
        assert np.array_equal(a0[17:23], a1[17:23]), key
        assert_fp32_sums_close(r1, r0)
        assert_fp32_sums_close(a1, a0)


@pytest.mark.parametrize("N", [64, 128])
def test_compensated_x4_matches_plain_compensated_bit_for_bit(N):
    """The compensated FP32 step in the x4 kernel (every variant) against
    step_kahan: identical fields and compensation words (the download returns
    hi - comp), SO rows to FP32-summation rounding, extrema exact; tuning
    leaves the state unchanged."""
    import ctypes
    import inputs
    PL = gpu()
    from phinum_gb300 import _lib as L
    phi_i, pi_i = inputs.lattice_fields(N, 1, 70, phi0=6 ** 0.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    lat = PL.Lattice(PL.Params(N=N, precision=2))
    nv = ctypes.c_int()
    L.check(lat.lib.phn_num_variants(lat.h, ctypes.byref(nv)))
    lat.close()
    assert nv.value >= 2
    out = {}
    for variant in [None] + list(range(nv.value)):
        lat = PL.Lattice(PL.Params(N=N, precision=2))
        if variant is None:
            L.check(lat.lib.phn_set_path(lat.h, L.PATH_PLAIN))
        else:
            L.check(lat.lib.phn_set_variant(lat.h, variant))
        lat.upload(phi, pi)
        rows = lat.run_loop(120, 0.5)
        lat.evolve(7)
        out[variant] = (rows,) + lat.download()
        lat.close()
    r0, f0, p0 = out[None]
    for key, (r1, f1, p1) in out.items():
        assert np.array_equal(f0, f1) and np.array_equal(p0[N * N:-N * N], p1[N * N:-N * N]), key
        assert np.array_equal(r0[:, 17:23], r1[:, 17:23]), key
        assert_fp32_sums_close(r1, r0)
    lat = PL.Lattice(PL.Params(N=N, precision=2))
    lat.upload(phi, pi)
    lat.evolve(3)
    before = lat.download()
    v, ms = ctypes.c_int(), ctypes.c_double()
    L.check(lat.lib.phn_autotune(lat.h, 3, ctypes.byref(v), ctypes.byref(ms)))
    after = lat.download()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1][N * N:-N * N], after[1][N * N:-N * N])
    assert v.value >= -1
    lat.close()


@pytest.mark.parametrize("precision", [1, 2])
def test_islands_fp32_with_a_spanning_cluster(precision):
    """FP32 (and compensated) fields at 128^3 with a mask over half the
    lattice, so that one cluster spans the box: labels and sizes equal the
    oracle's BFS on the same (FP32-valued) fields, energies within FP32
    rounding (the per-site terms are FP32 for FP32 fields, the per-island sums
    FP64)."""
    import inputs
    PL = gpu()
    N = 128
    phi_i, pi_i = inputs.lattice_fields(N, 1, 12)
    phi32, pi32 = phi_i.astype(np.float32).astype(np.float64), pi_i.astype(np.float32).astype(np.float64)
    phi, pi = O.to_ref_layout(phi32), O.to_ref_layout(pi32)
    thr = float(np.quantile(np.sqrt(phi32 ** 2 + pi32 ** 2), 0.5))
    lat = PL.Lattice(PL.Params(N=N, precision=precision))
    lat.upload(phi, pi)
    lab, recs = lat.full_analysis(thr)
    lat.close()
    olab, orecs = O.islands(O.Params(N=N), phi, pi, thr)
    assert np.array_equal(lab, olab)
    I = {k: i for i, k in enumerate(O.ISLAND_FIELDS)}
    assert np.array_equal(recs[:, I["size"]], orecs[:, I["size"]])
    assert recs[:, I["size"]].max() > 0.3 * N ** 3  # the spanning cluster
    for k in ("pot_en", "kin_en", "grad_en"):
        np.testing.assert_allclose(recs[:, I[k]], orecs[:, I[k]], rtol=2e-5, atol=1e-6 * np.abs(orecs[:, I[k]]).max())
    np.testing.assert_allclose(recs[:, I["av_phi"]], orecs[:, I["av_phi"]], rtol=1e-5, atol=1e-6)
    assert np.array_equal(np.abs(recs[:, I["peak_value"]]), np.abs(orecs[:, I["peak_value"]]))


def _cudart():
    import ctypes.util
    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart")):
        if not name:
            continue
        for cand in (name, os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", name)):
            try:
                return ctypes.CDLL(cand)
            except OSError:
                pass
    pytest.skip("libcudart not found for the device-to-host check")


@pytest.mark.parametrize("precision,N", [(1, 128), (0, 64), (2, 96), (1, 100)])
def test_islands_device_records_equal_host_records(precision, N):
    """phn_islands_device leaves the same records on the device that
    phn_islands copies to the host (tiled and untiled labellings, FP32, FP64
    and compensated fields), and the labels it leaves behind answer lookups
    like phn_islands'."""
    import inputs
    from phinum_gb300 import _lib as L
    PL = gpu()
    phi_i, pi_i = inputs.lattice_fields(N, 1, 12)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    thr = float(np.quantile(np.sqrt(phi_i ** 2 + pi_i ** 2), 0.6))
    lat = PL.Lattice(PL.Params(N=N, precision=precision))
    lat.upload(phi, pi)
    lab, recs = lat.full_analysis(thr)
    n, dptr = lat.full_analysis_device(thr)
    assert n == recs.shape[0] and n > 0 and dptr
    got = np.zeros_like(recs)
    rt = _cudart()
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(got.ctypes.data, ctypes.c_void_p(dptr), got.nbytes, 2) == 0  # device to host
    assert np.array_equal(got[:, :2], recs[:, :2]) and np.array_equal(got[:, 8:], recs[:, 8:])
    np.testing.assert_allclose(got[:, 2:8], recs[:, 2:8], rtol=1e-12, atol=1e-300)
    pos = np.flatnonzero(lab >= 0)[:: max(1, (lab >= 0).sum() // 1000)].astype(np.int64)
    isl = np.zeros(pos.size, dtype=np.int32)
    L.check(lat.lib.phn_islands_lookup(lat.h, pos.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), pos.size,
                                       isl.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    assert np.array_equal(isl, lab[pos])
    lat.close()


def test_records_into_a_caller_buffer_and_spectrum_timing():
    """full_analysis(out=...) writes the records into a caller-owned,
    page-locked buffer (phn_pin_host): the same islands as a fresh array
    (ids, sizes, peaks exact; the FP64 sums add block partials in arrival
    order, so they agree to rounding); phn_spectrum_timing reports the device
    time of the last spectrum call's transforms and binning."""
    import inputs
    from phinum_gb300 import _lib as L
    PL = gpu()
    N = 64
    phi_i, pi_i = inputs.lattice_fields(N, 1, 12)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    thr = float(np.quantile(np.sqrt(phi_i ** 2 + pi_i ** 2), 0.6))
    lat = PL.Lattice(PL.Params(N=N, precision=1))
    lat.upload(phi, pi)
    _, recs = lat.full_analysis(thr, labels=False)
    buf = np.zeros((recs.shape[0] + 5, len(L.ISLAND_FIELDS)))
    L.check(lat.lib.phn_pin_host(buf.ctypes.data, buf.nbytes))
    try:
        _, got = lat.full_analysis(thr, labels=False, out=buf)
        assert got.shape == recs.shape and np.shares_memory(got, buf)
        exact = [0, 1, 2, 7, 8, 9]
        assert np.array_equal(got[:, exact], recs[:, exact])
        assert np.all(np.abs(got - recs) <= 1e-12 * np.abs(recs).max(axis=0))
        with pytest.raises(ValueError):
            lat.full_analysis(thr, labels=False, out=np.zeros((4, 3)))
    finally:
        lat.lib.phn_unpin_host(buf.ctypes.data)
    lat.correlation_functions()
    t, b = lat.spectrum_timing()
    assert t > 0 and b > 0
    lat.spectrum_uniform(64)
    t, b = lat.spectrum_timing()
    assert t > 0 and b > 0
    lat.close()


@pytest.mark.parametrize("N", [24, 47, 100])
def test_islands_at_edges_that_are_not_powers_of_two(N):
    """Rows that straddle the 32-site warp segments of the labelling (its
    run links and x-wrap unions) and index division by an edge that is not a
    power of two: labels, sizes and seeds equal the oracle's for both masks,
    z open and periodic, FP64 and (reference mask) FP32 fields."""
    import inputs
    PL = gpu()
    phi_i, pi_i = inputs.lattice_fields(N, 1, 31)
    phi32, pi32 = phi_i.astype(np.float32).astype(np.float64), pi_i.astype(np.float32).astype(np.float64)
    op = O.Params(N=N)
    for precision, (ph, pp) in ((0, (phi_i, pi_i)), (1, (phi32, pi32))):
        phi, pi = O.to_ref_layout(ph), O.to_ref_layout(pp)
        thr = float(np.quantile(np.sqrt(ph ** 2 + pp ** 2), 0.45))
        rho = O.averages(op, phi, pi)[O.AVG["energy"]]
        lat = PL.Lattice(PL.Params(N=N, precision=precision))
        lat.upload(phi, pi)
        for mode, t in ((0, thr), (1, 1.2 * rho)):
            if precision and mode:
                continue  # the FP32 energy mask rounds differently near the threshold
            for zper in (0, 1):
                lab, recs = lat.full_analysis(t, mode=mode, z_periodic=bool(zper))
                olab, orecs = O.islands(op, phi, pi, t, mode=mode, zper=zper)
                assert np.array_equal(lab, olab), (precision, mode, zper)
                assert np.array_equal(recs[:, 1], orecs[:, 1]) and np.array_equal(recs[:, 9], orecs[:, 9])
        lat.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_single_precision_host_layout(precision):
    """phn_upload_f32 / phn_download_f32 (the reference's single-precision
    build, pseudo_double = float): the same reference layout with float
    elements.  Float inputs give the device the same state as their double
    values; the float download is the double download rounded; ghost slabs
    as phn_download's."""
    import inputs
    PL = gpu()
    N = 32
    phi_i, pi_i = inputs.lattice_fields(N, 1, 13)
    phi32 = O.to_ref_layout(phi_i).astype(np.float32)
    pi32 = O.to_ref_layout(pi_i).astype(np.float32)
    out = []
    for host in (np.float32, np.float64):
        lat = PL.Lattice(PL.Params(N=N, precision=precision))
        lat.upload(phi32.astype(host), pi32.astype(host))
        lat.evolve(5)
        out.append((lat.download(), lat.download(np.float32)))
        lat.close()
    (d64_a, d32_a), (d64_b, d32_b) = out
    for x, y in zip(d64_a, d64_b):
        assert np.array_equal(x, y)
    for x, y in zip(d32_a, d32_b):
        assert np.array_equal(x, y)
    slab = N * N
    assert np.array_equal(d32_a[0], d64_a[0].astype(np.float32))
    assert np.array_equal(d32_a[1][slab:-slab], d64_a[1][slab:-slab].astype(np.float32))
