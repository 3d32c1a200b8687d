"""The FP64 kernels' constant division, restated on the host
(tests/divide_check.c), against IEEE division: one Markstein correction
after a faithful first quotient -- RN(a RN(1/b)) for 6 Nc, 24 Nc, 120 Nc^2
(whose reciprocals are within 2^-54), fma(a, y_h, a y_l) with a two-word
reciprocal for every other divisor -- returns a / b bit for bit over the
range the kernels use it for.  test_gpu_divide.py checks the device code."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")
def test_constant_division_restatement_is_ieee(tmp_path):
    exe = str(tmp_path / "divide_check")
    # no contraction: every fma here is written out, every product rounds
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", os.path.join(ROOT, "tests", "divide_check.c"), "-o", exe,
           "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe, "100000"], capture_output=True, text=True, timeout=300).stdout
    m = re.search(r"divisors (\d+) operands (\d+) misses (\d+) near_divisors_not_near (\d+)", out)
    assert m, out
    nb, done, misses, not_near = map(int, m.groups())
    assert nb == 92 and done > 5_000_000, out
    assert misses == 0 and not_near == 0, out
