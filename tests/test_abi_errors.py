"""Host-side checks of the C ABI, on the CPU: NULL handles and bad
parameters return PHN_ERR_* status codes (with a message) before any CUDA
call, so these run without a GPU."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def L():
    from phinum_gb300 import build
    build.build()
    from phinum_gb300 import _lib
    _lib.load()
    return _lib


def create_status(L, **kw):
    from phinum_gb300 import lattice as PL
    p = PL.Params(**kw)
    h = ctypes.c_void_p()
    return L.load().phn_create(ctypes.byref(p.c()), ctypes.byref(h))


@pytest.mark.parametrize("kw,code", [
    (dict(N=1), "ERR_INVALID"),
    (dict(N=4096), "ERR_INVALID"),
    (dict(N=8, Nc=9), "ERR_UNSUPPORTED"),
    (dict(N=8, theory=6), "ERR_INVALID"),
    (dict(N=8, theory=2, m_sqr=0.0), "ERR_INVALID"),
    (dict(N=8, theory=5, p_mono=0.0), "ERR_INVALID"),
    (dict(N=8, theory=0, kappa=0.0), "ERR_INVALID"),
    (dict(N=8, precision=3), "ERR_UNSUPPORTED"),  # FP32 pairs: the adjoint's forward only
    (dict(N=8, precision=4), "ERR_INVALID"),
    (dict(N=8, a=0.0), "ERR_INVALID"),
    (dict(N=8, expansion=2), "ERR_INVALID"),
    (dict(N=8, expansion=1, H0=0.0), "ERR_INVALID"),
    (dict(N=8, expansion=1, H0=0.1, T0=-20.0), "ERR_INVALID"),
])
def test_create_rejects_bad_parameters(L, kw, code):
    assert create_status(L, **kw) == getattr(L, code)
    assert L.load().phn_last_error()  # a message says why


def test_null_handles_are_status_codes(L):
    lib = L.load()
    d = ctypes.c_double()
    i = ctypes.c_int()
    buf = (ctypes.c_double * 8)()
    calls = [
        lambda: lib.phn_upload(None, buf, buf),
        lambda: lib.phn_download(None, buf, buf),
        lambda: lib.phn_upload_f32(None, None, None),
        lambda: lib.phn_download_f32(None, None, None),
        lambda: lib.phn_evolve(None, 1),
        lambda: lib.phn_reset(None),
        lambda: lib.phn_time(None, ctypes.byref(d), ctypes.byref(i)),
        lambda: lib.phn_conformal_time(None, ctypes.byref(d), ctypes.byref(d)),
        lambda: lib.phn_adjoint_forward(None, buf, buf, ctypes.byref(d)),
        lambda: lib.phn_adjoint_backward(None, None, None, None),
        lambda: lib.phn_adjoint_set_forward_precision(None, 0),
        lambda: lib.phn_adjoint_info(None, None, None, None),
        lambda: lib.phn_spectrum_timing(None, ctypes.byref(d), ctypes.byref(d)),
    ]
    for c in calls:
        assert c() == L.ERR_INVALID
    assert lib.phn_destroy(None) == L.OK  # like free(NULL)


def test_noalloc_scratch_limit_is_exactly_n_1024(L):
    """The allocation-free averages hold ceil(N/32) * ceil(N/8) block records
    in a fixed array of 4096: the size check (host only, before any CUDA call)
    must pass every N <= 1024 and reject every larger N.  With NULL field
    pointers an accepted size then fails on the NULL check instead."""
    from phinum_gb300 import lattice as PL
    lib = L.load()
    out = L.PhnAverages()
    for N in list(range(2, 80)) + list(range(980, 1100)):
        p = PL.Params(N=N, precision=1)
        assert lib.phn_volume_averages_noalloc(ctypes.byref(p.c()), None, None, None, ctypes.byref(out)) == \
            L.ERR_INVALID
        assert (b"N <= 1024" in lib.phn_last_error()) == (N > 1024), N
        assert ((N + 31) // 32) * ((N + 7) // 8) <= 4096 or N > 1024


def test_ensemble_and_adjoint_parameter_checks_on_the_host(L):
    """The one-clock rule of the ensemble (a, dt, T0 and the box shared:
    all static, or all expanding with one H0) and the adjoint's theory/Nc
    rules are checked on the host before any CUDA call."""
    from phinum_gb300 import lattice as PL
    lib = L.load()

    def ens(*ps):
        arr = (L.PhnParams * len(ps))(*[p.c() for p in ps])
        h = ctypes.c_void_p()
        return lib.phn_ensemble_create(arr, len(ps), ctypes.byref(h))

    static, exp1 = PL.Params(N=32, precision=1), PL.Params(N=32, precision=1, expansion=1, H0=0.05)
    assert ens(static, exp1) == L.ERR_INVALID
    assert ens(exp1, PL.Params(N=32, precision=1, expansion=1, H0=0.06)) == L.ERR_INVALID
    assert ens(static, PL.Params(N=32, precision=1, T0=1.0)) == L.ERR_INVALID
    assert ens(PL.Params(N=32, precision=1, theory=2, m_sqr=1.0)) == L.ERR_UNSUPPORTED
    h = ctypes.c_void_p()
    for p in (PL.Params(N=16, precision=0, Nc=2), PL.Params(N=16, precision=0, theory=3, m_sqr=1.0)):
        assert lib.phn_adjoint_create(ctypes.byref(p.c()), 10, 5, 0.6, ctypes.byref(h)) == L.ERR_UNSUPPORTED
    assert lib.phn_adjoint_create(ctypes.byref(static.c()), 10, 3, 0.6, ctypes.byref(h)) == L.ERR_INVALID
