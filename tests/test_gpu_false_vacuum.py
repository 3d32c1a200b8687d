"""The run loop's false-vacuum break (main.cpp:85-89) driven through the
library on the GPU: each row from phn_volume_averages at the reference's TSO
cadence, phn_false_vacuum_decayed on it, phn_evolve(1) between rows -- the
call sequence of the reference-side adapter.  The loop must stop at the step
where the reference's own loop stopped (fixtures tests/golden/fvd/: a tilted
well whose <V> turns negative at step 151, and a NaN in Pi that reaches phi
with the first drift, stopping at step 10), with the rows of the reference
(FP64 sums 1e-11 relative, extrema of finite rows exact; FP32 rows 2e-5 and
compensated FP32 rows 5e-6 of each column's largest value: the rows' per-site
terms are FP32 in both)."""
import numpy as np
import pytest

import run_loops
from test_false_vacuum import FVD, fvd_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,rtol", [(0, 1e-11), (1, 2e-5), (2, 5e-6)])
@pytest.mark.parametrize("name", FVD)
def test_library_loop_stops_where_the_reference_loop_stops(name, precision, rtol):
    from phinum_gb300 import lattice as PL

    d, Phi, Pi = fvd_case(name)
    p = PL.Params(**{**d["params"], "precision": precision})
    with PL.Lattice(p) as lat:
        lat.upload(Phi, Pi)
        lat.reset()
        rows, stop = run_loops.loop_until_decayed(
            lat.time, lambda: lat.volume_averages(allow_nonfinite=True), lambda: lat.evolve(1),
            run_loops.decayed_by_library(lat.lib, p.theory), int(d["steps"]), float(d["tso"]))
    ref = d["rows"]
    assert stop == int(d["stop"]) > 0
    rows = np.asarray(rows)
    assert rows.shape[0] == ref.shape[0]
    assert np.array_equal(rows[:, 0], ref[:, 0])
    # <V> crosses zero: FP32 errors are measured against each column's scale
    for c in range(1, 17):
        scale = np.nanmax(np.abs(ref[:, c])) if np.isfinite(ref[:, c]).any() else 0.0
        np.testing.assert_allclose(rows[:, c], ref[:, c], rtol=rtol if precision == 0 else 0.0,
                                   atol=1e-300 if precision == 0 else rtol * scale, equal_nan=True)
    finite = np.isfinite(ref[:, 15])
    if precision == 0:
        assert np.array_equal(rows[finite, 17:23], ref[finite, 17:23])
    # NaN reaches the rows exactly where it reaches the reference's
    assert np.array_equal(np.isnan(rows[:, 15]), np.isnan(ref[:, 15]))
