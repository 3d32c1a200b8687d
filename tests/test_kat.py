"""Analytic known-answer tests of the oracle (tests/kat.py): the exact
discrete plane wave, second-order convergence to the homogeneous-field ODE,
and the energy error's order (second for the synchronized energy, first for
the reference's own staggered Energy, which pairs phi_n with pi_{n-1/2})."""
import numpy as np
import pytest

import inputs
import kat
from oracle import oracle as O


def test_plane_wave_is_exact():
    N, a, dt = 16, 0.25, 0.08
    p = O.Params(**kat.wave_params(N, a, dt))
    phi, pi = O.to_ref_layout(kat.plane_wave(N, a)), O.to_ref_layout(np.zeros((N, N, N)))
    steps = 1000
    O.evolve(p, phi, pi, steps)
    want_phi, want_pi = kat.plane_wave_exact(N, a, a * dt, steps)
    assert np.abs(O.from_ref_layout(phi, N)[0] - want_phi).max() <= 1e-11
    assert np.abs(O.from_ref_layout(pi, N)[0] - want_pi).max() <= 1e-10


def leapfrog_uniform(h: float, T: float, f0: float) -> float:
    p = O.Params(**kat.phi6_params(4, 0.25, h))
    phi, pi = O.to_ref_layout(np.full((4, 4, 4), f0)), O.to_ref_layout(np.zeros((4, 4, 4)))
    O.evolve(p, phi, pi, int(round(T / h)))
    return float(O.from_ref_layout(phi, 4)[0].mean())


def test_homogeneous_field_converges_at_second_order():
    pytest.importorskip("scipy")
    T, f0 = 20.0, 2.0
    exact = kat.ode_reference(f0, T)
    errs = [abs(leapfrog_uniform(h, T, f0) - exact) for h in (0.04, 0.02, 0.01)]
    assert errs[1] < 3e-4
    for e1, e2 in zip(errs, errs[1:]):
        assert 3.7 < e1 / e2 < 4.3


def energy_errors(h: float, T: float = 4.0):
    """(synchronized, staggered) relative energy error after T."""
    N = 16
    ph, pp = inputs.lattice_fields(N, 1, 5, phi0=1.0, amp_phi=0.6, amp_pi=0.6)
    p = O.Params(**kat.phi6_params(N, 0.25, h))
    phi, pi = O.to_ref_layout(ph), O.to_ref_layout(pp)
    E0 = O.averages(p, phi, pi)[O.AVG["energy"]]
    clock = O.evolve(p, phi, pi, int(round(T / h)))
    e_stag = O.averages(p, phi, pi)[O.AVG["energy"]]
    phi_n, pi_half = phi.copy(), pi.copy()
    O.evolve(p, phi, pi, 1, clock)
    e_sync = O.averages(p, phi_n, 0.5 * (pi_half + pi))[O.AVG["energy"]]
    return abs(e_sync - E0) / abs(E0), abs(e_stag - E0) / abs(E0)


def test_energy_error_order():
    a, b = energy_errors(0.02), energy_errors(0.01)
    assert 3.6 < a[0] / b[0] < 4.4   # synchronized: O(h^2)
    assert 1.6 < a[1] / b[1] < 2.6   # staggered (the reference's diagnostic): O(h)
    assert b[0] < 1e-3
