"""Island tracking over a run (phn_tracker_*), the host bookkeeping on CPU:
fed with the oracle's island labelling of the oracle's (reference-exact
FP64) fields, the tracker must reproduce the reference's own Full_Analysis
history (fixture tests/golden/track/, made by make_golden.py from the pinned
reference): indices, statuses, disp flags, history lengths, centres and sizes
exactly; float statistics to 1e-10 relative (summation order).  Plus the
rules the run does not reach (oscillon status, history cap, ties in the
volume sort, merging), on synthetic records."""
import json
import os

import numpy as np
import pytest

import inputs
from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "track")


def load(name):
    with np.load(os.path.join(HERE, name + ".npz"), allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


def tracker():
    from phinum_gb300 import lattice as PL
    return PL.Tracker()


def compare_call(d, c, got, cell):
    o0, o1 = int(d["offs"][c]), int(d["offs"][c + 1])
    ref = d["ints"][o0:o1]
    assert got.shape[0] == ref.shape[0], (c, got.shape[0], ref.shape[0])
    H = got[:, 4:].reshape(-1, 5, 8)
    iv = np.zeros((got.shape[0], 14), dtype=np.int64)
    iv[:, :4] = got[:, :4].astype(np.int64)
    iv[:, 4:9] = H[:, :, 1].astype(np.int64)
    iv[:, 9:14] = np.rint(H[:, :, 2] / cell).astype(np.int64)
    assert np.array_equal(iv, ref), c
    fl = H[:, :, [0, 3, 4, 5, 6, 7]]
    np.testing.assert_allclose(fl.sum(axis=(0, 1)), d["sums"][c], rtol=1e-10, atol=1e-9)
    if f"floats_{c}" in d:
        ref_f = d[f"floats_{c}"]
        np.testing.assert_allclose(fl, ref_f, rtol=1e-10, atol=1e-10 * max(1.0, np.abs(ref_f).max()))


def test_tracking_matches_reference_full_analysis():
    from phinum_gb300 import lattice as PL
    d = load("n24_phi6")
    pd = d["params"]
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    N, thr, every = p.N, float(d["thres"]), int(d["every"])
    phi_i, pi_i = inputs.lattice_fields(N, 1, int(d["seed"]), phi0=6 ** 0.5)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    clock = O.Clock(p)
    cell = p.a ** 3
    T = PL.Tracker()
    seen_status = set()
    for c in range(int(d["ncalls"])):
        labels, recs = O.islands(p, phi, pi, thr)
        centers = T.centers()
        ci = labels[centers] if centers.size else np.zeros(0, dtype=np.int32)
        T.update_records(clock.tau, recs, ci)
        got = T.islands()
        compare_call(d, c, got, cell)
        seen_status |= set(got[:, 1].astype(int))
        O.evolve(p, phi, pi, every, clock)
    assert seen_status >= {0, 1}
    T.close()


def rec(size, peak_pos, pot=1.0, grad=1.0, a=0.25):
    r = np.zeros(10)
    r[1], r[2], r[3], r[5], r[7], r[8] = size, size * a * a * a, pot, grad, peak_pos, 1.0
    return r


def test_rules_on_synthetic_records():
    T = tracker()
    # call 1: three new islands in seed order
    T.update_records(0.0, np.array([rec(5, 100), rec(9, 200), rec(5, 300)]), np.zeros(0))
    a = T.islands()
    assert list(a[:, 0]) == [0, 1, 2] and list(a[:, 2]) == [1, 1, 1]
    # call 2: the centres of islands 0 and 2 fall in one island, island 1's
    # centre left the mask; one new island.  Sorting puts 9 first, then the
    # two 5s: the first of those claims the shared island, the other merges.
    from phinum_gb300 import _lib as L
    comps = np.array([rec(7, 110), rec(4, 999)])
    owner = T.update_records(1.0, comps, np.array([0, -1, 0]))
    a = T.islands()
    r = T.islands(L.TRACK_RETIRED)
    assert list(r[:, 0]) == [1]
    assert a.shape[0] == 2 and a[0, 0] in (0, 2) and a[1, 0] == 3
    assert list(owner) == [0, 1]
    # a bubble (GradEn + PotEn < 0) is reported and gets status 1
    comps = np.array([rec(7, 120, pot=-3.0), rec(4, 999)])
    T.update_records(2.0, comps, np.array([0, 1]))
    b = T.islands(L.TRACK_BUBBLES)
    a = T.islands()
    assert b.shape[0] == 1 and a[0, 1] == 1 and a[1, 1] == 0
    # oscillon: alive longer than 40 time units; history capped at 5 entries
    for k, tau in enumerate((10.0, 20.0, 30.0, 45.0)):
        T.update_records(tau, np.array([rec(7, 120), rec(4, 999)]), np.array([0, 1]))
    a = T.islands()
    assert a[0, 3] == 5 and a[0, 1] == 2
    # entries at t = 0, 1, 2, 10, 20, 30, 45; kept: the first two and the last three
    times = a[0, 4:].reshape(5, 8)[:, 0]
    assert list(times) == [0.0, 1.0, 20.0, 30.0, 45.0]
    osc = np.zeros(3)
    L.check(T.lib.phn_tracker_oscillons(T.h, 8, 0.25, 1.0, osc.ctypes.data_as(L._PD)))
    assert osc[1] > 0
    hr, hr0 = np.zeros(40000, dtype=np.int32), np.zeros(40000, dtype=np.int32)
    L.check(T.lib.phn_tracker_add_stat(T.h, 0.5, 1.0, hr.ctypes.data_as(L._PI), hr0.ctypes.data_as(L._PI)))
    assert hr.sum() == 2
    # bad centre index
    with pytest.raises(L.PhnError):
        T.update_records(50.0, np.array([rec(7, 120)]), np.array([5, 0]))
    T.close()
