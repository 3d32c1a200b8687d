"""The island labelling's shortcuts on the host, from the header the kernels
include (phinum_gb300/csrc/ccl_math.h): the multiply-high division of site
indices by the lattice edge is exact, and the FP32 decision of the
reference mask agrees with the reference's FP64 test wherever it decides
(tests/ccl_math_check.cpp)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_ccl_math_on_host(tmp_path):
    exe = str(tmp_path / "ccl_math_check")
    # no FP contraction: the reference's FP64 test rounds each operation
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "phinum_gb300", "csrc"),
           os.path.join(ROOT, "tests", "ccl_math_check.cpp"), "-o", exe, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300).stdout
    m = re.search(r"divn checked (\d+) mismatches (\d+)", out)
    assert m and int(m.group(1)) > 1_000_000 and int(m.group(2)) == 0, out
    m = re.search(r"bracket checked (\d+) decided (\d+) wrong (\d+)", out)
    assert m, out
    total, decided, wrong = map(int, m.groups())
    assert wrong == 0 and decided > 0, out
    # three quarters of the draws put the threshold within 2^-18 of the sum
    # on purpose; thresholds drawn at random are nearly all decided in FP32
    m = re.search(r"random thresholds (\d+) decided (\d+)", out)
    assert m and int(m.group(2)) > 0.99 * int(m.group(1)), out
