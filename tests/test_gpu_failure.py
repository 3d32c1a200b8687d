"""Failure detection on the GPU without a fault: a bounded device wait on a
barrier that nothing completes gives up, the host reads PHN_ERR_TIMEOUT, and
the context stays usable (the same handle then evolves exactly as a fresh
one)."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_stays_usable():
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    N = 128
    phi_i, pi_i = inputs.lattice_fields(N, 1, 77, phi0=6 ** 0.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    with PL.Lattice(PL.Params(N=N, precision=1)) as lat:
        lat.upload(phi, pi)
        assert lat.lib.phn_wait_selftest(lat.h, 10000) == L.ERR_TIMEOUT
        assert b"gave up" in lat.lib.phn_last_error()
        assert lat.lib.phn_wait_selftest(lat.h, 0) == L.ERR_INVALID
        lat.evolve(10)  # the TMA step's own bounded waits report nothing
        a = lat.download()
    with PL.Lattice(PL.Params(N=N, precision=1)) as lat:
        lat.upload(phi, pi)
        lat.evolve(10)
        b = lat.download()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1][N * N:-N * N], b[1][N * N:-N * N])

