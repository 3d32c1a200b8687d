"""Checkpoint files through a handle: phn_save_config writes the reference's
bytes for the handle's state (FP64: the fields bit-identical to the
reference's after the same steps) and the moment file; phn_load_config
restores the state exactly and returns the time stamp."""
import hashlib

import numpy as np
import pytest

import inputs
from oracle import oracle as O
from test_config_io import CASES, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", [c for c in CASES if c.endswith("f64")])
def test_save_config_matches_reference_bytes(name, tmp_path):
    from phinum_gb300 import lattice as PL
    d = load(name)
    pd = d["params"]
    seed = {"n8_f64": 11, "n8_nc2_f64": 12}[name]
    phi_i, pi_i = inputs.lattice_fields(pd["N"], pd["Nc"], seed, phi0=6 ** 0.5)
    with PL.Lattice(PL.Params(precision=0, **pd)) as lat:
        lat.upload(O.to_ref_layout(phi_i, pd["Nc"]), O.to_ref_layout(pi_i, pd["Nc"]))
        lat.reset()
        lat.evolve(3)
        lat.save_config(3, str(tmp_path))
        raw = (tmp_path / "field-3-0.out").read_bytes()
        assert hashlib.sha256(raw).hexdigest() == str(d["sha"])
        assert (tmp_path / "moment-3.out").read_text() == str(d["moment"])
        phi, pi = lat.download()
    with PL.Lattice(PL.Params(precision=0, **pd)) as lat2:
        t0 = lat2.load_config(3, str(tmp_path))
        phi2, pi2 = lat2.download()
    sl = slice(pd["Nc"] * pd["N"] ** 2, -pd["Nc"] * pd["N"] ** 2)
    assert np.array_equal(phi, phi2) and np.array_equal(pi[sl], pi2[sl])
    assert t0 == float(str(d["moment"]))
