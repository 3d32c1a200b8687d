"""The reference-side adapter (phinum_gb300/adapter/phinum_dynamics.cpp).

1. It compiles inside the reference's own translation unit, for every theory,
   in the static and the expanding box, double and float builds.
2. It runs: tests/adapter_run.cpp is the reference's run sequence (main.cpp:
   Prepare_Output, set-up, per run fix_tadpole + SetInitialConditions, the
   loop of main.cpp:77-90 with its false-vacuum break), built twice from the
   reference's sources -- once with the reference's own reset / evolve /
   Print_AveragesExtrema / Print_fp, once with the adapter's drop-ins linked
   against a CPU stand-in of the library (tests/adapter_standin.c, the oracle
   behind the same C ABI).  Both runs must write the same SO-<run>.txt and
   Distrib-<run>-<t>.txt files, byte for byte.
3. It refuses a multi-rank run (each rank then holds one z-slab) instead of
   reading past the rank's arrays.

Needs the reference tree (present where the build runs); skipped elsewhere.
"""
import concurrent.futures as cf
import filecmp
import os
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.ref_dir()
HAVE_REF = os.path.isfile(os.path.join(REF, "dynamics.cpp"))
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference tree not present")
INCLUDES = ["-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "oracle"), "-I", REF,
            "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "phinum_gb300", "adapter")]


@needs_ref
@pytest.mark.parametrize("precision", [0, -1])
@pytest.mark.parametrize("expansion", [0, 1])
@pytest.mark.parametrize("theory", [0, 1, 2, 3, 4, 5])
def test_adapter_compiles_in_reference_tu(theory, expansion, precision):
    if precision == -1 and theory != 0:
        pytest.skip("the single-precision build is checked with theory 0")
    cmd = ["g++", "-std=gnu++14", "-fsyntax-only", "-w", f"-DPHN_REF_THEORY={theory}",
           f"-DPHN_REF_PRECISION={precision}", f"-DPHN_REF_EXPANSION={expansion}", *INCLUDES,
           os.path.join(ROOT, "tests", "adapter_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


PHI6 = "Kappa=1.7320508075688772 phi0=2.449489742783178"
# the tilted well with a strong tilt: <V> turns negative mid-run, and the
# false_vacuum_decayed() break ends the loop there
TILT = "Mass_Mode=-1 Lambda_Mode=1 h=0.6 phi0=0.8"
# scale2 above the largest lattice momentum: every spectrum bin holds signal
# (a cut-off spectrum has bins of pure transform round-off, where the
# reference's FFT and the oracle's differ in the printed digits)
RUNS = {
    "t0_static_two_runs": (0, 0, f"N=12 runs=2 seed=7 TMax=6 TSO=0.25 TMO=1 {PHI6} Noise=0.05 scale2=100"),
    "t0_expanding": (0, 1, f"N=12 runs=1 seed=7 TMax=6 TSO=0.25 TMO=1 {PHI6} Noise=0.05 scale2=100"),
    "t1_static_decays": (1, 0, f"N=16 runs=1 seed=5 TMax=8 TSO=0.2 TMO=0.5 {TILT} Noise=0.05 scale2=100"),
    "t1_expanding": (1, 1, f"N=12 runs=1 seed=5 TMax=6 TSO=0.2 TMO=0.5 {TILT} Noise=0.05 scale2=100"),
}
FLAGS = ["-std=gnu++14", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w"]


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stderr[-3000:])


@pytest.fixture(scope="module")
def binaries(tmp_path_factory):
    """The CPU stand-in library and, per (theory, expansion), the reference's
    loop with its own functions and with the adapter; plus the adapter built
    against an MPI stand-in that reports two ranks."""
    d = str(tmp_path_factory.mktemp("adapter"))
    _compile(["gcc", "-std=c99", "-shared", "-fPIC", "-O2", "-ffp-contract=off", "-fno-fast-math",
              "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests", "adapter_standin.c"), os.path.join(ROOT, "oracle", "phinum_oracle.c"),
              "-o", os.path.join(d, "libphinum_gpu.so"), "-lm"])
    src = os.path.join(ROOT, "tests", "adapter_run.cpp")
    link = ["-L", d, "-lphinum_gpu", f"-Wl,-rpath,{d}"]
    jobs, out = [], {}
    for t, e in sorted({(t, e) for t, e, _ in RUNS.values()}):
        base = [*FLAGS, f"-DPHN_REF_THEORY={t}", f"-DPHN_REF_EXPANSION={e}", *INCLUDES, src]
        out[(t, e, 0)] = os.path.join(d, f"ref_{t}{e}")
        out[(t, e, 1)] = os.path.join(d, f"adapter_{t}{e}")
        jobs.append(["g++", *base, "-DPHN_ADAPTER=0", "-o", out[(t, e, 0)]])
        jobs.append(["g++", *base, "-DPHN_ADAPTER=1", "-o", out[(t, e, 1)], *link])
    out["two_ranks"] = os.path.join(d, "adapter_two_ranks")
    jobs.append(["g++", *FLAGS, "-DPHN_REF_THEORY=0", "-DPHN_SHIM_NODES=2", "-DPHN_ADAPTER=1", *INCLUDES, src,
                 "-o", out["two_ranks"], *link])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(_compile, jobs))
    return out


def _run(binary, args, cwd):
    os.makedirs(cwd)
    r = subprocess.run([binary, *args.split()], cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return os.path.join(cwd, "output", "1")


@needs_ref
@pytest.mark.parametrize("name", sorted(RUNS))
def test_adapter_run_writes_the_reference_files(binaries, tmp_path, name):
    theory, expansion, args = RUNS[name]
    ref = _run(binaries[(theory, expansion, 0)], args, str(tmp_path / "reference"))
    gpu = _run(binaries[(theory, expansion, 1)], args, str(tmp_path / "adapter"))
    files = sorted(os.listdir(ref))
    assert files == sorted(os.listdir(gpu))
    assert sum(f.startswith("Distrib") for f in files) >= 2 and any(f.startswith("SO") for f in files)
    with open(os.path.join(ref, "SO-1.txt")) as f:
        assert len(f.read().splitlines()) >= 10  # the loop ran (no immediate false-vacuum break)
    _, mismatch, errors = filecmp.cmpfiles(ref, gpu, files, shallow=False)
    assert not mismatch and not errors, mismatch + errors


@needs_ref
def test_adapter_refuses_a_multi_rank_run(binaries, tmp_path):
    """With two ranks each rank's Phi/Pi hold N/2 z-slabs: the adapter stops
    with a message before phn_create / phn_upload could read past them."""
    r = subprocess.run([binaries["two_ranks"], "guard_only", "N=8"], cwd=str(tmp_path), capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1
    assert "one rank" in r.stderr and "2 rank(s)" in r.stderr
