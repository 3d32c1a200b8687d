"""Analytic known-answer tests of the CUDA path through the C ABI
(tests/kat.py): the exact discrete plane wave in every precision, the
homogeneous-field ODE at second order (FP64), and the synchronized energy
error at second order (FP64).

Tolerances: FP64 1e-11 (phi) / 1e-10 (pi) after 1000 steps, as the oracle;
FP32 2e-5 and compensated FP32 5e-6 of the wave's amplitude 0.7 (a numpy
FP32 restatement of the same run is off by 1.2e-6 / 3.7e-6)."""
import numpy as np
import pytest

import inputs
import kat
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def lattice(**kw):
    from phinum_gb300 import lattice as PL
    return PL.Lattice(PL.Params(**kw))


@pytest.mark.parametrize("precision,tol_phi,tol_pi", [(0, 1e-11, 1e-10), (1, 2e-5, 2e-5), (2, 5e-6, 5e-6)])
@pytest.mark.parametrize("N", [16, 64])
def test_plane_wave_is_exact(N, precision, tol_phi, tol_pi):
    a, dt, steps = 0.25, 0.08, 1000
    with lattice(precision=precision, **kat.wave_params(N, a, dt)) as lat:
        lat.upload(O.to_ref_layout(kat.plane_wave(N, a)), O.to_ref_layout(np.zeros((N, N, N))))
        lat.evolve(steps)
        phi, pi = lat.download()
    want_phi, want_pi = kat.plane_wave_exact(N, a, a * dt, steps)
    assert np.abs(O.from_ref_layout(phi, N)[0] - want_phi).max() <= tol_phi
    assert np.abs(O.from_ref_layout(pi, N)[0] - want_pi).max() <= tol_pi


def test_homogeneous_field_converges_at_second_order():
    pytest.importorskip("scipy")
    T, f0 = 20.0, 2.0
    exact = kat.ode_reference(f0, T)
    errs = []
    for h in (0.04, 0.02, 0.01):
        with lattice(precision=0, **kat.phi6_params(32, 0.25, h)) as lat:
            lat.upload(O.to_ref_layout(np.full((32, 32, 32), f0)), O.to_ref_layout(np.zeros((32, 32, 32))))
            lat.evolve(int(round(T / h)))
            phi, _ = lat.download()
        f = O.from_ref_layout(phi, 32)[0]
        assert np.all(f == f.flat[0])  # a uniform field stays uniform
        errs.append(abs(float(f.flat[0]) - exact))
    assert errs[1] < 3e-4
    for e1, e2 in zip(errs, errs[1:]):
        assert 3.7 < e1 / e2 < 4.3


def test_synchronized_energy_error_is_second_order():
    N, T = 32, 4.0
    ph, pp = inputs.lattice_fields(N, 1, 5, phi0=1.0, amp_phi=0.6, amp_pi=0.6)
    errs = []
    for h in (0.02, 0.01):
        with lattice(precision=0, **kat.phi6_params(N, 0.25, h)) as lat:
            lat.upload(O.to_ref_layout(ph), O.to_ref_layout(pp))
            E0 = lat.volume_averages()[O.AVG["energy"]]
            lat.evolve(int(round(T / h)))
            phi_n, pi_half = lat.download()
            lat.evolve(1)
            _, pi_next = lat.download()
        # pi_n = (pi_{n-1/2} + pi_{n+1/2}) / 2; the energy of (phi_n, pi_n) through the oracle's averages
        p = O.Params(**kat.phi6_params(N, 0.25, h))
        E = O.averages(p, phi_n, 0.5 * (pi_half + pi_next))[O.AVG["energy"]]
        errs.append(abs(E - E0) / abs(E0))
    assert 3.6 < errs[0] / errs[1] < 4.4
