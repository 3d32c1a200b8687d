"""Momentum-space filter (apply_filter, filter.cpp:53-133): the oracle's
restatement against the reference's own output (tests/golden/filter/, made
by make_golden.py with the pinned reference); the transforms are the
oracle's DFT, so agreement is to rounding (1e-13 of the largest value)."""
import glob
import json
import os

import numpy as np
import pytest

import inputs
from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "filter")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "*.npz")))


def load(name):
    with np.load(os.path.join(HERE, name + ".npz"), allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


def table():
    """The tabulated window of the fixtures (make_golden.py filter_table)."""
    return np.exp(-np.arange(25000) * 0.001) * (1.0 + 0.1 * np.cos(np.arange(25000) * 0.01))


def inputs_of(d):
    pd = d["params"]
    phi, pi = inputs.lattice_fields(pd["N"], pd["Nc"], int(d["seed"]), phi0=6 ** 0.5)
    return O.to_ref_layout(phi, pd["Nc"]), O.to_ref_layout(pi, pd["Nc"])


def test_fixtures_present():
    assert len(CASES) >= 5


@pytest.mark.parametrize("name", CASES)
def test_oracle_filter_matches_reference(name):
    d = load(name)
    pd = d["params"]
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi, pi = inputs_of(d)
    ophi, opi = O.apply_filter(p, phi, pi, float(d["r"]), int(d["which"]), table(), float(d["dp"]))
    sl = slice(pd["Nc"] * pd["N"] ** 2, -pd["Nc"] * pd["N"] ** 2)
    for got, ref in ((ophi[sl], d["phi"][sl]), (opi[sl], d["pi"][sl])):
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    # the filter changed the fields
    assert np.abs(d["phi"][sl] - phi[sl]).max() > 1e-3
