"""Momentum-space filter on the GPU (phn_apply_filter) against the
reference's own apply_filter output: FP64 within 1e-12 of the largest
value (cuFFT and CUDA's exp/sin/cos round differently), FP32 within 1e-5."""
import numpy as np
import pytest

from test_filter import CASES, inputs_of, load, table

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_gpu_filter_matches_reference(name, precision, tol):
    from phinum_gb300 import lattice as PL
    d = load(name)
    pd = d["params"]
    phi, pi = inputs_of(d)
    with PL.Lattice(PL.Params(precision=precision, **pd)) as lat:
        lat.upload(phi, pi)
        lat.apply_filter(float(d["r"]), int(d["which"]), table(), float(d["dp"]))
        gphi, gpi = lat.download()
    sl = slice(pd["Nc"] * pd["N"] ** 2, -pd["Nc"] * pd["N"] ** 2)
    for got, ref in ((gphi[sl], d["phi"][sl]), (gpi[sl], d["pi"][sl])):
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_gpu_filter_rejects_bad_arguments():
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    with PL.Lattice(PL.Params(N=8)) as lat:
        assert lat.lib.phn_apply_filter(lat.h, 0.5, 7, None, 0, 0.0) == L.ERR_INVALID
        assert lat.lib.phn_apply_filter(lat.h, 0.5, L.FILTER_TABLE, None, 0, 0.0) == L.ERR_INVALID
