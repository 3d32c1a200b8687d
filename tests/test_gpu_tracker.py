"""Island tracking on the GPU (phn_tracker_update: GPU labelling, centre
lookups, host bookkeeping) over an FP64 run, against the reference's own
Full_Analysis history (fixture tests/golden/track/): integer data and the
labels (island_analysis::b) exactly, float statistics to 1e-10 relative."""
import hashlib

import numpy as np
import pytest

import inputs
from oracle import oracle as O
from test_tracker import compare_call, load

pytestmark = pytest.mark.gpu


def test_gpu_tracking_matches_reference_full_analysis():
    from phinum_gb300 import lattice as PL
    d = load("n24_phi6")
    pd = d["params"]
    N, thr, every = pd["N"], float(d["thres"]), int(d["every"])
    phi_i, pi_i = inputs.lattice_fields(N, 1, int(d["seed"]), phi0=6 ** 0.5)
    with PL.Lattice(PL.Params(precision=0, **pd)) as lat, PL.Tracker() as T:
        lat.upload(O.to_ref_layout(phi_i), O.to_ref_layout(pi_i))
        lat.reset()
        for c in range(int(d["ncalls"])):
            lab = T.update(lat, thr, labels=True)
            compare_call(d, c, T.islands(), 0.25 ** 3)
            assert hashlib.sha256(lab.astype("<i4").tobytes()).hexdigest() == str(d["labels_sha"][c]), c
            lat.evolve(every)


def test_gpu_tracking_fp32_runs():
    from phinum_gb300 import lattice as PL
    N = 32
    phi_i, pi_i = inputs.lattice_fields(N, 1, 9, phi0=6 ** 0.5)
    thr = float(np.quantile(np.sqrt(phi_i ** 2 + pi_i ** 2), 0.95))
    with PL.Lattice(PL.Params(N=N, precision=1)) as lat, PL.Tracker() as T:
        lat.upload(O.to_ref_layout(phi_i), O.to_ref_layout(pi_i))
        lat.reset()
        for c in range(10):
            lab = T.update(lat, thr, labels=True)
            a = T.islands()
            # labels are positions in found_islands; every island owns sites
            assert lab.max() == a.shape[0] - 1 and set(np.unique(lab[lab >= 0])) == set(range(a.shape[0]))
            lat.evolve(20)
