"""Hand-written adjoint (phn_adjoint_*): gradients against central finite
differences of the forward objective (FP64), and FP32 gradients against the
FP64 adjoint.

Tolerances: FP64 adjoint vs FD, relative 1e-6 per direction (FD step 1e-5,
O(h^2) truncation); FP32 vs FP64 adjoint, relative L2 error of the field
gradient 2e-3 on short runs."""
import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SQ6 = 6 ** 0.5


def setup(N, seed, theory=0):
    from phinum_gb300 import lattice as PL
    phi0 = SQ6 if theory == 0 else -SQ6
    phi, pi = inputs.lattice_fields(N, 1, seed, phi0=phi0)
    kw = dict(theory=0, kappa=3 ** 0.5) if theory == 0 else dict(theory=1, mass_mode=-1, lambda_mode=1, h=0.3)
    return kw, O.to_ref_layout(phi), O.to_ref_layout(pi)


def direction(N, seed):
    rng = np.random.default_rng(seed)
    v = O.to_ref_layout(rng.standard_normal((N, N, N)))
    return v / np.linalg.norm(v[N * N:-N * N])


@pytest.mark.parametrize("expansion", [0, 1])
@pytest.mark.parametrize("theory", [0, 1])
def test_fp64_adjoint_matches_finite_differences(theory, expansion):
    """Static and expanding box (H0 = 0.05 from T0 = 2: the scale factor
    grows from 1.095 to 1.105 over the run)."""
    from phinum_gb300 import lattice as PL
    N, steps, every = 16, 40, 10
    kw, phi, pi = setup(N, 7 + theory, theory)
    if expansion:
        kw = dict(kw, expansion=1, H0=0.05, T0=2.0)
    p = PL.Params(N=N, precision=0, **kw)
    with PL.Adjoint(p, steps, every) as adj:
        J0 = adj.forward(phi, pi)
        dphi, dpi, g = adj.backward()
        eps = 1e-5
        sl = slice(N * N, -N * N)
        for k in range(3):
            v = direction(N, 100 + k)
            fd = (adj.forward(phi + eps * v, pi) - adj.forward(phi - eps * v, pi)) / (2 * eps)
            ad = float(np.dot(dphi[sl], v[sl]))
            assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(J0)), (k, ad, fd)
            fdp = (adj.forward(phi, pi + eps * v) - adj.forward(phi, pi - eps * v)) / (2 * eps)
            adp = float(np.dot(dpi[sl], v[sl]))
            assert abs(adp - fdp) <= 1e-6 * max(abs(fdp), 1e-3 * abs(J0)), (k, adp, fdp)
        # homogeneous shift of the initial phi
        one = np.ones_like(phi)
        fd = (adj.forward(phi + eps * one, pi) - adj.forward(phi - eps * one, pi)) / (2 * eps)
        assert abs(g[0] - fd) <= 1e-6 * abs(fd), (g[0], fd)
    # coupling: c6 = 1/(720 Kappa^2) (theory 0) or h (theory 1), by re-running with it perturbed
    def J_at(delta):
        if theory == 0:
            c6 = 1.0 / (720 * kw["kappa"] ** 2) + delta
            q = PL.Params(N=N, precision=0, **dict(kw, kappa=(1.0 / (720 * c6)) ** 0.5))
        else:
            q = PL.Params(N=N, precision=0, **dict(kw, h=kw["h"] + delta))
        with PL.Adjoint(q, steps, every) as a2:
            return a2.forward(phi, pi)
    epsc = 1e-8 if theory == 0 else 1e-6
    fd = (J_at(epsc) - J_at(-epsc)) / (2 * epsc)
    ad = g[1] if theory == 0 else g[2]
    assert abs(ad - fd) <= 2e-6 * abs(fd), (ad, fd)


@pytest.mark.parametrize("expansion", [0, 1])
def test_fp32_adjoint_close_to_fp64_adjoint(expansion):
    from phinum_gb300 import lattice as PL
    N, steps, every = 32, 100, 50
    kw, phi, pi = setup(N, 21)
    if expansion:
        kw = dict(kw, expansion=1, H0=0.05, T0=2.0)
    out = {}
    for prec in (0, 1):
        with PL.Adjoint(PL.Params(N=N, precision=prec, **kw), steps, every) as adj:
            J = adj.forward(phi, pi)
            out[prec] = (J,) + adj.backward()
    sl = slice(N * N, -N * N)
    J64, d64, p64, g64 = out[0]
    J32, d32, p32, g32 = out[1]
    assert abs(J32 - J64) <= 1e-4 * abs(J64)
    assert np.linalg.norm(d32[sl] - d64[sl]) <= 2e-3 * np.linalg.norm(d64[sl])
    assert np.linalg.norm(p32[sl] - p64[sl]) <= 2e-3 * np.linalg.norm(p64[sl])
    assert abs(g32[0] - g64[0]) <= 2e-3 * abs(g64[0])
    assert abs(g32[1] - g64[1]) <= 2e-3 * abs(g64[1])


def test_backward_is_deterministic_and_forward_matches_evolve():
    from phinum_gb300 import lattice as PL
    N, steps, every = 32, 60, 20
    kw, phi, pi = setup(N, 5)
    p = PL.Params(N=N, precision=1, **kw)
    with PL.Adjoint(p, steps, every) as adj:
        adj.forward(phi, pi)
        a = adj.backward()
        adj.forward(phi, pi)
        b = adj.backward()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    with pytest.raises(Exception):
        PL.Adjoint(p, 61, 20)


def test_fp64_forward_fp32_adjoint_within_1e4_of_fp64_adjoint():
    """phn_adjoint_set_forward_precision(PHN_FP64) under an FP32 adjoint: the
    forward runs the FP64 step kernels (J is the FP64 adjoint's, bit for bit),
    checkpoints and reverse sweep stay FP32; the field gradient is within
    1e-4 (relative L2) of the FP64 adjoint's.  Back to FP32 it is the plain
    FP32 adjoint again, bit for bit; an FP64 adjoint refuses the switch."""
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    N, steps, every = 32, 200, 50
    kw, phi, pi = setup(N, 23)
    sl = slice(N * N, -N * N)
    with PL.Adjoint(PL.Params(N=N, precision=0, **kw), steps, every) as adj:
        J64 = adj.forward(phi, pi)
        d64, p64, g64 = adj.backward()
        with pytest.raises(L.PhnError) as e:
            L.check(adj.lib.phn_adjoint_set_forward_precision(adj.h, 1))
        assert e.value.code == L.ERR_UNSUPPORTED
    with PL.Adjoint(PL.Params(N=N, precision=1, **kw), steps, every, forward_precision=0) as adj:
        Jm = adj.forward(phi, pi)
        dm, pm, gm = adj.backward()
        assert Jm == J64
        assert np.linalg.norm(dm[sl] - d64[sl]) <= 1e-4 * np.linalg.norm(d64[sl])
        assert np.linalg.norm(pm[sl] - p64[sl]) <= 1e-4 * np.linalg.norm(p64[sl])
        assert abs(gm[0] - g64[0]) <= 1e-4 * abs(g64[0])
        assert abs(gm[1] - g64[1]) <= 1e-4 * abs(g64[1])
        L.check(adj.lib.phn_adjoint_set_forward_precision(adj.h, 1))
        adj.forward(phi, pi)
        back = adj.backward()
    with PL.Adjoint(PL.Params(N=N, precision=1, **kw), steps, every) as adj:
        adj.forward(phi, pi)
        plain = adj.backward()
    for x, y in zip(back, plain):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("expansion", [0, 1])
def test_pair_forward_fp32_adjoint_within_1e4_of_fp64_adjoint(expansion):
    """phn_adjoint_set_forward_precision(PHN_FP32_PAIR): the forward in FP32
    pairs (double-float arithmetic), FP32 checkpoints and reverse sweep.  J is
    the FP64 adjoint's to 1e-8 relative (the pair state carries ~48 bits; its
    Laplacian sums the high words' differences plainly, which leaves the pair
    trajectory ~1e-6 from FP64's after 1000 steps, against ~5e-5 for FP32),
    the gradients within 1e-4 of the FP64 adjoint's; back to FP32 the plain
    FP32 adjoint returns, bit for bit."""
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    N, steps, every = 32, 200, 50
    kw, phi, pi = setup(N, 23)
    if expansion:  # the pair step takes each step's scale factor like the FP64 one
        kw = dict(kw, expansion=1, H0=0.05, T0=2.0)
    sl = slice(N * N, -N * N)
    with PL.Adjoint(PL.Params(N=N, precision=0, **kw), steps, every) as adj:
        J64 = adj.forward(phi, pi)
        d64, p64, g64 = adj.backward()
    with PL.Adjoint(PL.Params(N=N, precision=1, **kw), steps, every, forward_precision=L.FP32_PAIR) as adj:
        Jp = adj.forward(phi, pi)
        dp, pp, gp = adj.backward()
        assert abs(Jp - J64) <= 1e-8 * abs(J64)
        assert np.linalg.norm(dp[sl] - d64[sl]) <= 1e-4 * np.linalg.norm(d64[sl])
        assert np.linalg.norm(pp[sl] - p64[sl]) <= 1e-4 * np.linalg.norm(p64[sl])
        assert abs(gp[0] - g64[0]) <= 1e-4 * abs(g64[0])
        assert abs(gp[1] - g64[1]) <= 1e-4 * abs(g64[1])
        L.check(adj.lib.phn_adjoint_set_forward_precision(adj.h, 1))
        adj.forward(phi, pi)
        back = adj.backward()
    with PL.Adjoint(PL.Params(N=N, precision=1, **kw), steps, every) as adj:
        adj.forward(phi, pi)
        plain = adj.backward()
    for x, y in zip(back, plain):
        assert np.array_equal(x, y)


def test_adjoint_against_central_differences_20_directions_64():
    """The gradient check of the adjoint configuration at 64^3 x 200 steps
    (checkpoints every 50): central differences of the FP64 forward, step
    h = 1e-3, along 20 seeded random unit directions of the initial phi.  The
    FP64 adjoint agrees to 1e-5 per direction and the FP32 adjoint with its
    forward in FP32 pairs to 1e-4; the all-FP32 adjoint's error is reported
    beside them (its forward's FP32 rounding, amplified by the sigmoid)."""
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    N, steps, every, h, ndir = 64, 200, 50, 1e-3, 20
    kw, phi, pi = setup(N, 41)
    sl = slice(N * N, -N * N)
    grads = {}
    for name, prec, fwd in (("fp64", 0, None), ("pair", 1, L.FP32_PAIR), ("fp32", 1, None)):
        with PL.Adjoint(PL.Params(N=N, precision=prec, **kw), steps, every, forward_precision=fwd) as adj:
            adj.forward(phi, pi)
            grads[name] = adj.backward()[0][sl]
    rng = np.random.default_rng(99)
    err = {k: [] for k in grads}
    with PL.Adjoint(PL.Params(N=N, precision=0, **kw), steps, every) as adj:
        for _ in range(ndir):
            v = np.zeros_like(phi)
            v[sl] = rng.standard_normal(N ** 3)
            v /= np.linalg.norm(v[sl])
            fd = (adj.forward(phi + h * v, pi) - adj.forward(phi - h * v, pi)) / (2 * h)
            for k, g in grads.items():
                err[k].append(abs(float(np.dot(g, v[sl])) - fd) / abs(fd))
    print({k: max(v) for k, v in err.items()})
    assert max(err["fp64"]) <= 1e-5
    assert max(err["pair"]) <= 1e-4
