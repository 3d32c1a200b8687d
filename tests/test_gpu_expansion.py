"""The expanding box (the reference's `expansion 1`: radiation era,
a = sqrt(1 + 2 H_0 tau), kick and drift in conformal time) on the GPU.

The e* fixtures in tests/golden/ come from the reference's own expansion
build; the FP64 field, row and island checks of test_gpu_parity.py run over
them too.  Here: the scale-factor column and the conformal clock (exact: the
same FP64 expressions on the host), the FP32 and compensated paths (folded
couplings) within the FP32 tolerances, and the x4 / TMA kernels bit-identical
to the plain FP32 kernel under expansion.
"""
import ctypes

import numpy as np
import pytest

import fixtures
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EXP_CASES = [n for n in fixtures.names() if n.startswith("e")]
SF_COL = 25


def start(d, precision, **kw):
    from phinum_gb300 import lattice as PL
    p = PL.Params(precision=precision, a=d["a"], dt=d["dt"], **d["params"], **kw)
    lat = PL.Lattice(p)
    phi_i, pi_i = fixtures.inputs_for(d)
    lat.upload(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    return lat, p


def test_expansion_fixtures_present():
    assert len(EXP_CASES) >= 6


@pytest.mark.parametrize("name", EXP_CASES)
def test_scale_factor_column_and_conformal_clock(name):
    d = fixtures.load(name)
    lat, p = start(d, 0)
    rows = lat.run_loop(d["steps"], d["tso"])
    assert np.array_equal(rows[:, SF_COL], d["rows"][:, SF_COL])
    assert rows[-1, SF_COL] > 1.0
    op = O.Params(a=d["a"], dt=d["dt"], **d["params"])
    oracle_clock = O.Clock(op)
    phi_i, pi_i = fixtures.inputs_for(d)
    O.evolve(op, O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc), d["steps"], oracle_clock)
    assert lat.conformal_time() == (oracle_clock.tau_c, oracle_clock.sf)
    assert lat.volume_averages()[SF_COL] == oracle_clock.sf
    lat.close()


@pytest.mark.parametrize("precision,atol", [(1, 2e-4), (2, 2e-5)])
@pytest.mark.parametrize("name", ["e0_n8_nc2", "e2_n8", "e3_n8", "e5_n8"])
def test_fp32_expanding_fields_close(name, precision, atol):
    d = fixtures.load(name)
    lat, p = start(d, precision)
    last = max(fixtures.checkpoints(d))
    lat.evolve(last)
    phi, pi = lat.download()
    np.testing.assert_allclose(O.from_ref_layout(phi, p.N, p.Nc), d[f"phi_{last}"], rtol=0, atol=atol)
    np.testing.assert_allclose(O.from_ref_layout(pi, p.N, p.Nc), d[f"pi_{last}"], rtol=0, atol=atol)
    a = lat.volume_averages()
    ref = d[f"avg_{last}"]
    for col in ("energy", "interaction", "phi2", "pi2", "charge"):
        j = O.AVG[col]
        assert abs(a[j] - ref[j]) <= 1e-4 * max(1.0, abs(ref[j])), col
    lat.close()


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("N,theory", [(128, 0), (64, 1), (96, 4)])
def test_fast_paths_match_plain_under_expansion(N, theory, precision):
    """Every FP32 kernel takes the same couplings folded with the step's scale
    factor: the x4 variants and the TMA variants (FP32, N = 128) leave fields
    bit-identical to the plain kernel's; rows agree to FP32-summation
    rounding, extrema exactly."""
    import inputs
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    kw = {0: dict(theory=0), 1: dict(theory=1, mass_mode=-1, lambda_mode=1, h=0.12247),
          4: dict(theory=4, mass_mode=1, lambda_mode=1, g=0.5)}[theory]
    pp = dict(N=N, precision=precision, expansion=1, H0=0.05, T0=1.5, **kw)
    phi_i, pi_i = inputs.lattice_fields(N, 1, 80 + theory, phi0=(-1) ** theory * 1.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    lat = PL.Lattice(PL.Params(**pp))
    nv = ctypes.c_int()
    L.check(lat.lib.phn_num_variants(lat.h, ctypes.byref(nv)))
    lat.close()
    out = {}
    for variant in [None] + list(range(nv.value)):
        lat = PL.Lattice(PL.Params(**pp))
        if variant is None:
            L.check(lat.lib.phn_set_path(lat.h, L.PATH_PLAIN))
        else:
            L.check(lat.lib.phn_set_variant(lat.h, variant))
        lat.upload(phi, pi)
        rows = lat.run_loop(60, 0.3)
        lat.evolve(5)
        out[variant] = (rows,) + lat.download() + (lat.conformal_time(),)
        lat.close()
    r0, f0, p0, c0 = out[None]
    for key, (r1, f1, p1, c1) in out.items():
        assert np.array_equal(f0, f1) and np.array_equal(p0[N * N:-N * N], p1[N * N:-N * N]), key
        assert c0 == c1
        assert np.array_equal(r0[:, 17:23], r1[:, 17:23]), key
        assert np.array_equal(r0[:, SF_COL], r1[:, SF_COL]), key
        np.testing.assert_allclose(r0[:, 9:17], r1[:, 9:17], rtol=1e-6, atol=1e-9)


def test_expanding_box_errors_are_status_codes():
    """Bad H_0, expansion switch or T0 is refused; the ensemble and the adjoint
    take the expanding box (their own tests compare them with single lattices
    and finite differences), the ensemble only with one clock."""
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    for kw, code in ((dict(expansion=1, H0=0.0), L.ERR_INVALID), (dict(expansion=2), L.ERR_INVALID),
                     (dict(expansion=1, H0=0.1, T0=-20.0), L.ERR_INVALID)):
        with pytest.raises(L.PhnError) as e:
            PL.Lattice(PL.Params(N=8, **kw))
        assert e.value.code == code
    p = PL.Params(N=32, precision=1, expansion=1)
    PL.Ensemble([p, p]).close()
    PL.Adjoint(PL.Params(N=16, precision=0, expansion=1), 10, 5).close()
    with pytest.raises(L.PhnError) as e:
        PL.Ensemble([p, PL.Params(N=32, precision=1)])
    assert e.value.code == L.ERR_INVALID
