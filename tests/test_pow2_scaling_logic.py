"""The float64 row moments scale a row sum / a sum of squared deviations by
1/n or 1/(n*divisor); when that factor is a power of two the device code
moves the exponent field on the integer pipes instead of multiplying
(`mul_pow2` in xtensor_gb300/csrc/xtg_device.cuh), and the host encodes the
factor's exponent (`rdiv_e2` / `vfac_e2`, xtensor_gb300/csrc/xtg_assign.cpp).
Restated here step for step and checked bit for bit against the plain
multiplication, including the edges where the fast form must give way.
CPU only: this pins the logic; the GPU tests pin the kernels."""
from __future__ import annotations

import math

import numpy as np


def _encode(f: float) -> int:
    m, k = math.frexp(f)
    return k - 1 + 100000 if (m == 0.5 and -1000 < k - 1 < 1000) else 0


def _mul_pow2(v: float, f: float, e2: int) -> float:
    if e2:
        b = int(np.array(v, np.float64).view(np.int64))
        ef = (b >> 52) & 0x7FF
        e = ef + (e2 - 100000)
        if ef != 0 and ef != 0x7FF and 1 <= e <= 2046:
            return float(np.array(b + ((e2 - 100000) << 52), np.int64).view(np.float64))
    return v * f


def test_encoding():
    assert _encode(1.0 / 1024) == -10 + 100000
    assert _encode(1.0 / 3) == 0
    assert _encode(2.0**-20) == -20 + 100000
    assert _encode(float("inf")) == 0
    assert _encode(0.0) == 0


def test_exponent_move_is_the_multiplication():
    g = np.random.default_rng(11)
    vals = np.concatenate([g.standard_normal(2000) * 10.0 ** g.integers(-300, 300, 2000),
                           [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                            -1.7976931348623157e308, 1.0, -1.0, float("inf"), float("-inf"), float("nan")]])
    for k in (-1074, -1030, -200, -20, -10, -1, 0, 1, 10, 200, 1023):
        f = 2.0**k
        e2 = _encode(f)
        for v in vals:
            with np.errstate(over="ignore", under="ignore", invalid="ignore"):
                want = v * f  # infinities expected where the product overflows
            got = _mul_pow2(float(v), f, e2)
            if math.isnan(want):
                assert math.isnan(got)
            else:
                assert np.array(got).view(np.int64) == np.array(want).view(np.int64), (v, k)
