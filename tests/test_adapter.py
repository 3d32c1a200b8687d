"""The reference-side adapter (phinum_gb300/adapter/phinum_dynamics.cpp)
compiles inside the reference's own translation unit, for every theory, in
the static and the expanding box.
Needs the reference tree (present where the build runs); skipped elsewhere."""
import os
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.ref_dir()


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "dynamics.cpp")), reason="reference tree not present")
@pytest.mark.parametrize("precision", [0, -1])
@pytest.mark.parametrize("expansion", [0, 1])
@pytest.mark.parametrize("theory", [0, 1, 2, 3, 4, 5])
def test_adapter_compiles_in_reference_tu(theory, expansion, precision):
    if precision == -1 and theory != 0:
        pytest.skip("the single-precision build is checked with theory 0")
    cmd = ["g++", "-std=gnu++14", "-fsyntax-only", "-w", f"-DPHN_REF_THEORY={theory}",
           f"-DPHN_REF_PRECISION={precision}", f"-DPHN_REF_EXPANSION={expansion}",
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "oracle"),
           "-I", REF, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "phinum_gb300", "adapter"),
           os.path.join(ROOT, "tests", "adapter_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
