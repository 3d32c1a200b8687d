"""The reference-side adapter (phinum_gb300/adapter/phinum_dynamics.cpp)
running against the real library on the GPU, from a C++ harness that stands
in for the reference's globals (tests/adapter_gpu_harness.cpp; no reference
tree needed).  The harness runs the reference's sequence -- averages and the
island threshold, Full_Analysis's first labelling, then reset /
Print_AveragesExtrema / Full_Analysis every 5 steps / false_vacuum_decayed /
Print_fp / evolve -- on a 16^3 phi^6 lattice in FP64.  Checked against the
oracle: the final fields bit for bit, every SO row and every Distrib row to
the printed precision (six significant digits; FP64 sums agree to 1e-11), the
number of islands of the first labelling exactly."""
import os
import subprocess

import numpy as np
import pytest

import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def read_rows(path):
    with open(path) as f:
        return [np.array([float(x) for x in line.split()]) for line in f.read().splitlines() if line.strip()]


def close(a, b, scale):
    return np.allclose(a, b, rtol=2e-5, atol=1e-9 * scale)


def test_adapter_sequence_through_the_library(tmp_path):
    from phinum_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "harness")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "phinum_gb300", "adapter"),
                        os.path.join(ROOT, "tests", "adapter_gpu_harness.cpp"), "-L", os.path.dirname(lib),
                        "-lphinum_gpu", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    N, tso, tmo, tmax = 16, 0.2, 0.5, 2.0
    # zero-mean fields: the reference's threshold 2.57583 sqrt(<phi^2>)
    # (main.cpp:70) then leaves islands in the mask
    phi_i, pi_i = inputs.lattice_fields(N, 1, 77, phi0=0.0)
    phi, pi = O.to_ref_layout(phi_i), O.to_ref_layout(pi_i)
    phi.tofile(str(tmp_path / "phi.bin"))
    pi.tofile(str(tmp_path / "pi.bin"))
    r = subprocess.run([exe, f"N={N}", f"TMax={tmax}", f"TSO={tso}", f"TMO={tmo}"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    steps = int(r.stdout.split("steps=")[1].split()[0])
    assert steps == 100

    p = O.Params(N=N)
    # fields after the run: bit for bit
    ophi, opi = phi.copy(), pi.copy()
    O.evolve(p, ophi, opi, steps)
    gphi = np.fromfile(str(tmp_path / "fields_after.bin"))
    assert np.array_equal(gphi, ophi)

    # SO rows (time, phi, pi, phi2, pi2, phipi, phi4, phi6, E, V, Q, min, max, max|phi|)
    orows, _ = O.run_loop(p, phi.copy(), pi.copy(), steps, tso)
    cols = [0, 1, 5, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19]
    so = read_rows(str(tmp_path / "output" / "1" / "SO-1.txt"))
    assert len(so) == orows.shape[0]
    for g, o in zip(so, orows):
        assert close(g, o[cols], np.abs(o[cols]).max()), (g, o[cols])

    # Distrib files at the TMO stamps: bins with counts, the reference's columns
    dfiles = sorted(os.listdir(str(tmp_path / "output" / "1")))
    dfiles = [f for f in dfiles if f.startswith("Distrib")]
    stamps = [0, 25, 50, 75]  # steps of tau = 0, 0.5, 1, 1.5
    assert len(dfiles) == len(stamps), dfiles
    ph, pp = phi.copy(), pi.copy()
    clock = O.Clock(p)
    done = 0
    for s in stamps:
        O.evolve(p, ph, pp, s - done, clock)
        done = s
        F, K, Q, C = O.spectrum(p, ph, pp)
        want = O.spectrum_columns(p, F, K, Q, C)
        want = want[(C > 0) & (F != 0)]  # the printer skips empty bins
        t = s * 0.02
        name = "Distrib-1-%g.txt" % (0 if s == 0 else round(t, 10))
        got = read_rows(str(tmp_path / "output" / "1" / name))
        assert len(got) == want.shape[0], name
        for g, w in zip(got, want):
            assert close(g, w[:g.size], np.abs(w).max()), (name, g, w)

    # the first labelling's island count
    lines = open(str(tmp_path / "islands.txt")).read().split("\n")
    first = int(lines[0].split()[1])
    thr = float(r.stdout.split("thres=")[1].split()[0])
    _, recs = O.islands(p, phi, pi, thr)
    assert first == recs.shape[0] and first > 0
