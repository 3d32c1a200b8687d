"""phn_volume_averages_noalloc: averages of caller-owned device fields with
no allocation, for hosts that cannot call cudaMalloc where they need the
averages (a framework that owns all device memory, or a stream-ordered loop
in which a device-synchronising allocation is not allowed).

It runs the same fused observation kernel as phn_volume_averages, with its
block records in a fixed __device__ array, so its output must match the
handle-based entry point: extrema exactly, sums within the tolerances used
elsewhere (FP64 relative 1e-11; FP32 fields relative 2e-5).  Checked on two
calls in a row, since every call reuses the same scratch array, and across a
change of CUDA context, after which the array's address must be looked up
again.
"""
import ctypes
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXACT = [17, 18, 19, 20, 21, 22]  # min/max/max|phi| values and positions
SUMS = [1, 5, 9, 10, 11, 12, 13, 14, 15, 16, 23]


def noalloc_vs_handle(lat, p, rtol, calls=2):
    """Calls the allocation-free entry point `calls` times on the lattice's
    own device fields and checks each result against phn_volume_averages."""
    from phinum_gb300 import _lib as L

    ref = lat.volume_averages()
    d_phi, d_pi, st = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    L.check(lat.lib.phn_device_fields(lat.h, ctypes.byref(d_phi), ctypes.byref(d_pi), ctypes.byref(st)))
    lat.synchronize()
    for _ in range(calls):
        out = L.PhnAverages()
        L.check(lat.lib.phn_volume_averages_noalloc(ctypes.byref(p.c()), d_phi, d_pi, st, ctypes.byref(out)))
        got = np.frombuffer(bytes(out), dtype=np.float64)
        assert np.array_equal(got[EXACT], ref[EXACT])
        np.testing.assert_allclose(got[SUMS], ref[SUMS], rtol=rtol, atol=rtol * 1e-3)
        assert got[24] == 0.0
        assert got[0] == p.T0
    return ref


@pytest.mark.parametrize("precision,rtol", [(0, 1e-11), (1, 2e-5)])
@pytest.mark.parametrize("N,Nc", [(64, 1), (48, 2), (256, 1)])
def test_noalloc_matches_handle_averages_twice(precision, rtol, N, Nc):
    """At 256^3 every block marches 256 planes, so the per-thread compensated
    FP32 sums run over long columns."""
    from phinum_gb300 import lattice as PL

    p = PL.Params(N=N, Nc=Nc, precision=precision)
    phi_i, pi_i = inputs.lattice_fields(N, Nc, 31)
    with PL.Lattice(p) as lat:
        lat.upload(O.to_ref_layout(phi_i, Nc), O.to_ref_layout(pi_i, Nc))
        lat.evolve(9)
        noalloc_vs_handle(lat, p, rtol)


def test_noalloc_rejects_lattices_beyond_its_scratch():
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL

    lib = L.load()
    out = L.PhnAverages()
    p = PL.Params(N=1056, precision=1)
    r = lib.phn_volume_averages_noalloc(ctypes.byref(p.c()), None, None, None, ctypes.byref(out))
    assert r == L.ERR_INVALID
    assert b"N <= 1024" in lib.phn_last_error()
    p = PL.Params(N=64, precision=2)
    assert lib.phn_volume_averages_noalloc(ctypes.byref(p.c()), None, None, None, ctypes.byref(out)) == \
        L.ERR_UNSUPPORTED


def test_noalloc_expanding_box_uses_the_initial_scale_factor():
    """For the expanding box the allocation-free averages are those at
    tau = T0 (scale factor sqrt(1 + 2 H0 T0)): equal to the handle's averages
    right after upload, whose clock is at T0, time stamp included."""
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL

    N = 32
    p = PL.Params(N=N, precision=0, expansion=1, H0=0.05, T0=3.0)
    phi_i, pi_i = inputs.lattice_fields(N, 1, 32)
    with PL.Lattice(p) as lat:
        lat.upload(O.to_ref_layout(phi_i), O.to_ref_layout(pi_i))
        ref = lat.volume_averages()
        assert ref[25] == math.sqrt(1.0 + 2.0 * 0.05 * 3.0)
        d_phi, d_pi, st = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        L.check(lat.lib.phn_device_fields(lat.h, ctypes.byref(d_phi), ctypes.byref(d_pi), ctypes.byref(st)))
        lat.synchronize()
        out = L.PhnAverages()
        L.check(lat.lib.phn_volume_averages_noalloc(ctypes.byref(p.c()), d_phi, d_pi, st, ctypes.byref(out)))
        got = np.frombuffer(bytes(out), dtype=np.float64)
        assert got[0] == ref[0] == 3.0
        assert np.array_equal(got[EXACT], ref[EXACT])
        np.testing.assert_allclose(got[SUMS], ref[SUMS], rtol=1e-11, atol=1e-14)
        assert got[25] == ref[25]


# Run in a fresh process: it creates and destroys a second CUDA context.
CONTEXT_SCRIPT = r"""
import ctypes, sys
sys.path[:0] = [ROOT, ROOT + '/tests', ROOT + '/tests/golden']
import inputs
from oracle import oracle as O
from phinum_gb300 import lattice as PL
from test_zz_no_alloc import noalloc_vs_handle

cuda = ctypes.CDLL('libcuda.so.1')
assert cuda.cuInit(0) == 0
p = PL.Params(N=64, precision=1)
phi_i, pi_i = inputs.lattice_fields(64, 1, 33)
phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
# the runtime's primary context: set-up of the scratch address
lat_a = PL.Lattice(p)
lat_a.upload(phi, pi)
lat_a.evolve(5)
ref_a = noalloc_vs_handle(lat_a, p, 2e-5)
# a second context created with the driver API and made current: the cached
# address belongs to the primary context, so the call must look it up again
dev, ctx = ctypes.c_int(), ctypes.c_void_p()
assert cuda.cuDeviceGet(ctypes.byref(dev), 0) == 0
assert cuda.cuCtxCreate_v2(ctypes.byref(ctx), 0, dev) == 0
lat_b = PL.Lattice(p)
lat_b.upload(phi, pi)
lat_b.evolve(7)
noalloc_vs_handle(lat_b, p, 2e-5)
lat_b.close()
assert cuda.cuCtxDestroy_v2(ctx) == 0
# back on the primary context: looked up again, same results as before
ref_a2 = noalloc_vs_handle(lat_a, p, 2e-5)
assert (ref_a2[1:] == ref_a[1:]).all()
lat_a.close()
print('context switch ok')
"""


def test_noalloc_looks_the_scratch_up_again_in_another_context():
    """The scratch address is per CUDA context: after the calling thread's
    context changes (here to a context created with the driver API, as a
    device reset would also give), the next call looks the address up again
    and still matches the handle-based averages, and so does the first call
    back in the original context."""
    r = subprocess.run([sys.executable, "-c", CONTEXT_SCRIPT.replace("ROOT", repr(ROOT))], cwd=ROOT,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    assert "context switch ok" in r.stdout
