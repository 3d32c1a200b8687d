"""Initial conditions on the GPU (phn_initial_conditions) against the
reference's own SetInitialConditions output (fixtures) and the oracle.

Tolerances: FP64 fields within 1e-12 of the largest value (the stream and
mode assignment are exact; CUDA's log/sin/cos and cuFFT round differently
from the C library and FFTW); FP32 handles within 1e-6 relative."""
import numpy as np
import pytest

from oracle import oracle as O
from test_initial_conditions import IC_FIXTURES, load

pytestmark = pytest.mark.gpu


def gpu_ic(pd, ic, precision=0):
    from phinum_gb300 import lattice as PL
    with PL.Lattice(PL.Params(precision=precision, **pd)) as lat:
        lat.initial_conditions(**ic)
        return lat.download()


@pytest.mark.parametrize("name", IC_FIXTURES)
def test_gpu_initial_conditions_match_reference(name):
    d = load(name)
    pd = dict(d["params"])
    phi, pi = gpu_ic(pd, d["ic"])
    N, Nc = pd["N"], pd["Nc"]
    sl = slice(Nc * N * N, -Nc * N * N)
    assert np.abs(phi - d["phi"]).max() <= 1e-12 * np.abs(d["phi"]).max()
    assert np.abs(pi[sl] - d["pi"][sl]).max() <= 1e-12 * np.abs(d["pi"][sl]).max()
    phi32, pi32 = gpu_ic(pd, d["ic"], precision=1)
    assert np.abs(phi32 - d["phi"]).max() <= 1e-6 * np.abs(d["phi"]).max()
    assert np.abs(pi32[sl] - d["pi"][sl]).max() <= 1e-6 * np.abs(d["pi"][sl]).max()


@pytest.mark.parametrize("N,seed", [(32, 11), (64, 2026)])
def test_gpu_initial_conditions_match_oracle(N, seed):
    ic = dict(seed=seed, noise=3.0, scale2=6.2832, phi0=(6 ** 0.5, 0.0))
    pd = dict(N=N, Nc=1, theory=0, kappa=3 ** 0.5)
    phi, pi = gpu_ic(pd, ic)
    ophi, opi = O.initial_conditions(O.Params(N=N, kappa=3 ** 0.5), **ic)
    sl = slice(N * N, -N * N)
    assert np.abs(phi - ophi).max() <= 1e-12 * np.abs(ophi).max()
    assert np.abs(pi[sl] - opi[sl]).max() <= 1e-12 * np.abs(opi[sl]).max()


def test_gpu_initial_conditions_deterministic_and_seeded():
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    pd = dict(N=128, Nc=1, theory=0)
    a = gpu_ic(pd, dict(seed=5, noise=3.0, scale2=6.2832))
    b = gpu_ic(pd, dict(seed=5, noise=3.0, scale2=6.2832))
    c = gpu_ic(pd, dict(seed=6, noise=3.0, scale2=6.2832))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    with PL.Lattice(PL.Params(N=9)) as lat:
        with pytest.raises(L.PhnError) as e:
            lat.initial_conditions(seed=1)
        assert e.value.code == L.ERR_UNSUPPORTED


@pytest.mark.parametrize("mode", [
    dict(initialize=0, famp=0.5, lambda_=1.7, temperature=0.6, phi0s=0.9, pi0s=0.3),
    dict(initialize=1, QS=5.0, amplitude=0.8, noise=0.4, chi=1.3, phi0s=0.9),
    dict(initialize=2, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4, phi0s=0.9),
    dict(initialize=4, QS=5.0, scale2=7.0, noise=0.4, temperature=0.6, phi0=(1.0, 0.5)),
    dict(initialize=3, withcharge=1, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4, phi0=(1.0, 0.5)),
    dict(initialize=2, withcharge=1, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4, phi0s=0.9),
])
def test_gpu_initial_condition_modes_match_oracle_at_48(mode):
    """The other initialize switches and the charged stream at 48^3, Nc = 2
    (the charged variant's paired draws), against the oracle's restatement."""
    N = 48
    ic = dict(seed=77, **mode)
    pd = dict(N=N, Nc=2, theory=0, kappa=3 ** 0.5, m_sqr=0.7)
    phi, pi = gpu_ic(pd, ic)
    ophi, opi = O.initial_conditions(O.Params(N=N, Nc=2, kappa=3 ** 0.5, m_sqr=0.7), **ic)
    sl = slice(2 * N * N, -2 * N * N)
    assert np.abs(phi - ophi).max() <= 1e-12 * np.abs(ophi).max()
    assert np.abs(pi[sl] - opi[sl]).max() <= 1e-12 * np.abs(opi[sl]).max()
    assert np.std(ophi[sl]) > 1e-3


def test_gpu_initial_conditions_refuse_charged_initialize_4():
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    with PL.Lattice(PL.Params(N=8, Nc=2)) as lat:
        with pytest.raises(L.PhnError) as e:
            lat.initial_conditions(seed=1, initialize=4, withcharge=1)
        assert e.value.code == L.ERR_UNSUPPORTED
        with pytest.raises(L.PhnError) as e:
            lat.initial_conditions(seed=1, initialize=5)
        assert e.value.code == L.ERR_INVALID
