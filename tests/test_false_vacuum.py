"""false_vacuum_decayed() (fieldanalysis.cpp:887-893) and the run loop's
break on it (main.cpp:85-89), on the CPU: the library's
phn_false_vacuum_decayed (host code, no GPU involved) against the reference's
own function (live, where the reference pin is built) and its restatement in
the oracle, and the loop's stopping step on the oracle against the
reference's own loop (fixtures tests/golden/fvd/)."""
import ctypes
import math
import os

import numpy as np
import pytest

import run_loops
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
VALUES = [1.0, 0.0, -0.0, 5e-324, -5e-324, -1.0, -1e300, math.nan, -math.nan, math.inf, -math.inf, 1e300]
FVD = sorted(f[:-4] for f in os.listdir(os.path.join(HERE, "golden", "fvd")))


@pytest.fixture(scope="module")
def lib():
    from phinum_gb300 import build
    build.build()
    from phinum_gb300 import _lib
    return _lib.load()


def lib_decayed(lib, v, theory):
    from phinum_gb300 import _lib as L
    a = L.PhnAverages()
    a.interaction = v
    d = ctypes.c_int(-1)
    L.check(lib.phn_false_vacuum_decayed(ctypes.byref(a), theory, ctypes.byref(d)))
    return bool(d.value)


@pytest.mark.parametrize("theory", [0, 1, 2, 3, 4, 5])
def test_rule_matches_the_oracle_restatement(lib, theory):
    for v in VALUES:
        assert lib_decayed(lib, v, theory) == O.false_vacuum_decayed(v, theory), (theory, v)
    # theories 0, 1, 4 stop on a negative, NaN or infinite <V>; 2, 3, 5 never
    assert lib_decayed(lib, -1.0, theory) == (theory in (0, 1, 4))
    assert not lib_decayed(lib, -0.0, theory)


@pytest.mark.parametrize("theory", [0, 1, 2, 3, 4, 5])
def test_rule_matches_the_reference_function(lib, theory):
    path = O.ref_path(theory)
    if not os.path.exists(path):
        pytest.skip("reference pin not built")
    ref = ctypes.CDLL(path)
    ref.ref_false_vacuum_decayed.argtypes = [ctypes.c_double]
    ref.ref_false_vacuum_decayed.restype = ctypes.c_int
    for v in VALUES:
        assert lib_decayed(lib, v, theory) == bool(ref.ref_false_vacuum_decayed(v)), (theory, v)


def test_null_arguments(lib):
    from phinum_gb300 import _lib as L
    d = ctypes.c_int()
    assert lib.phn_false_vacuum_decayed(None, 0, ctypes.byref(d)) == L.ERR_INVALID
    assert lib.phn_false_vacuum_decayed(ctypes.byref(L.PhnAverages()), 0, None) == L.ERR_INVALID


def fvd_case(name):
    with np.load(os.path.join(HERE, "golden", "fvd", name + ".npz")) as z:
        d = {k: z[k] for k in z.files}
    import json
    import inputs
    d["params"] = json.loads(str(d["params"]))
    p = d["params"]
    phi_i, pi_i = inputs.lattice_fields(p["N"], p["Nc"], int(d["seed"]), phi0=float(d["phi0"]))
    Phi, Pi = O.to_ref_layout(phi_i, p["Nc"]), O.to_ref_layout(pi_i, p["Nc"])
    if int(d["nan_site"]) >= 0:
        Pi[int(d["nan_site"])] = np.nan
    return d, Phi, Pi


def check_rows(rows, ref_rows, rtol):
    assert len(rows) == len(ref_rows)
    rows = np.asarray(rows)
    assert np.array_equal(rows[:, 0], ref_rows[:, 0])  # LastSOoutput stamps
    np.testing.assert_allclose(rows[:, 1:17], ref_rows[:, 1:17], rtol=rtol, atol=1e-300, equal_nan=True)


@pytest.mark.parametrize("name", FVD)
def test_oracle_loop_stops_where_the_reference_loop_stops(lib, name):
    d, Phi, Pi = fvd_case(name)
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **d["params"])
    clock = O.Clock(p)
    phi, pi = Phi.copy(), Pi.copy()
    rows, stop = run_loops.loop_until_decayed(
        lambda: (clock.tau, clock.steps), lambda: O.averages(p, phi, pi, clock),
        lambda: O.evolve(p, phi, pi, 1, clock), run_loops.decayed_by_library(lib, p.theory),
        int(d["steps"]), float(d["tso"]))
    assert stop == int(d["stop"]) > 0
    check_rows(rows, d["rows"], 0.0)  # the oracle is the reference's arithmetic
