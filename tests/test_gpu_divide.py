"""The FP64 kernels' division by per-launch constants (div_by_near and div_by
in phn_internal.h: a multiply by a one- or two-word reciprocal, then one
residual correction) against IEEE division on the device."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("b", [6.0, 12.0, 18.0, 24.0, 3.0 ** 0.5, 120.0, 480.0, 720.0 * 3.0000000000000004, 0.0625,
                               0.7, 3.0, 1.0363397126425293, 1e-20, 3.7e25, 2.0 ** 101])
def test_fp64_constant_division_is_ieee(b):
    """The FP64 kernels divide by per-launch constants with a faithful first
    quotient (RN(a RN(1/b)) where b RN(1/b) is within 2^-54 of 1, else
    fma(a, y_h, a y_l) with the two-word reciprocal y_h + y_l) and one residual
    correction; every quotient must carry the
    bits of IEEE a / b (Markstein's theorem), over 2^25 device-drawn operands
    per divisor including near-midpoint quotients, zeros, subnormals,
    infinities and NaN.  Divisors outside [2^-100, 2^100] take IEEE division."""
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L
    with PL.Lattice(PL.Params(N=8)) as lat:
        bad = ctypes.c_longlong(-1)
        for seed in (1, 2):
            L.check(lat.lib.phn_divide_selftest(lat.h, b, 1 << 25, seed, ctypes.byref(bad)))
            assert bad.value == 0
