"""The integer-to-double rounding of the float64 row moments (`fix_to_double`
in xtensor_gb300/csrc/xtg_device.cuh: a 192-bit magnitude times 2^e2,
rounded to nearest even on the integer pipes), restated step for step and
checked against exact rounding (Python's Fraction -> float), across the
normal range, halfway patterns, the subnormal range (one rounding of the
64-bit window straight to the subnormal grid) and overflow.  CPU only: this
pins the logic; the GPU tests pin the kernels."""
from __future__ import annotations

import math
import random
import struct
from fractions import Fraction

M64 = (1 << 64) - 1


def _fix_to_double(q: int, neg: bool, e2: int) -> float:
    if q == 0:
        return -0.0 if neg else 0.0
    w = [q & M64, (q >> 64) & M64, (q >> 128) & M64, 0]
    top = q.bit_length() - 1
    sh = top - 63
    if sh <= 0:
        m, sticky = (w[0] << (-sh)) & M64, False
    else:
        wi, b = sh >> 6, sh & 63
        lo, hi = w[wi], w[wi + 1]
        m = ((lo >> b) | (hi << (64 - b))) & M64 if b else lo
        below = (lo << (64 - b)) & M64 if b else 0
        sticky = below != 0 or (wi >= 1 and w[0] != 0) or (wi == 2 and w[1] != 0)
    if top + e2 + 1023 < 1:  # below the normal range: one rounding to the 2^-1074 grid
        r = -(top - 63 + e2 + 1074)  # bits of the window below the grid (>= 12)
        if r >= 65:
            qv, rb, st = 0, 0, sticky or m != 0
        elif r == 64:
            qv, rb, st = 0, (m >> 63) & 1, sticky or ((m << 1) & M64) != 0
        else:
            qv, rb, st = m >> r, (m >> (r - 1)) & 1, sticky or ((m << (65 - r)) & M64) != 0
        if rb and (st or (qv & 1)):
            qv += 1
        v = math.ldexp(qv, -1074)
        return -v if neg else v
    mant = m >> 11
    rnd = (m >> 10) & 1
    sticky = sticky or (m & 0x3FF) != 0
    if rnd and (sticky or (mant & 1)):
        mant += 1
    e = top + e2
    if mant >> 53:
        mant >>= 1
        e += 1
    if e + 1023 > 2046:
        return -math.inf if neg else math.inf
    v = math.ldexp(mant, e - 52)
    return -v if neg else v


def _exact(q: int, neg: bool, e2: int) -> float:
    try:
        v = float(Fraction(q) * Fraction(2) ** e2)
    except OverflowError:
        v = math.inf
    return -v if neg else v


def test_rounds_once_everywhere():
    rnd = random.Random(3)
    for _ in range(60000):
        nb = rnd.choice([1, 5, 53, 54, 60, 64, 65, 100, 128, 150, 191])
        q = rnd.getrandbits(nb) | (1 << (nb - 1))
        if rnd.random() < 0.3:  # halfway and near-halfway patterns
            q = (q >> 12 << 12) | rnd.choice([0, 1 << 11, (1 << 11) + 1, (1 << 11) - 1])
        e2 = rnd.randint(-1200 - nb, 1100 - nb)
        neg = rnd.random() < 0.5
        got, want = _fix_to_double(q, neg, e2), _exact(q, neg, e2)
        assert got == want and math.copysign(1, got) == math.copysign(1, want), (q, e2, got, want)


def test_subnormal_edges():
    # halfway between two subnormals (ties to even), just above and below,
    # and the carry into the smallest normal
    for base in (0, 1, 2, 3, (1 << 52) - 1):
        for frac in (0, 1 << 62, (1 << 62) + 1, (1 << 62) - 1, (1 << 63) - 1):
            q = (base << 64) | frac  # value = q * 2^(-1074 - 64)
            if q == 0:
                continue
            assert _fix_to_double(q, False, -1074 - 64) == _exact(q, False, -1074 - 64), (base, frac)


def _fixed_mag(x: float, ef_max: int) -> int:
    """`fixed_mag`: |X| = |x| * 2^(1075 - ef_max) rounded half away from zero
    (twice the significand shifted down, plus one, halved)."""
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    hi, lo = b >> 32, b & 0xFFFFFFFF
    e = (hi >> 20) & 0x7FF
    m2 = ((((hi & 0xFFFFF) | (0x100000 if e else 0)) << 32) | lo) << 1
    sh = min(ef_max - (e if e else 1), 63)
    return ((m2 >> sh) + 1) >> 1


def test_fixed_point_elements_and_square_sums():
    """Each element becomes X = round(x * 2^(1075 - Ef)) (exact in the top
    binade, half away from zero below it), and a lane's sum of X^2 split as
    Xh^2 2^54 + 2 Xh Xl 2^27 + Xl^2 (|X| = Xh 2^27 + Xl, unsigned 32x32-bit
    products) is exact."""
    rnd = random.Random(5)
    for _ in range(3000):
        ef = rnd.randint(2, 2046)
        xs = []
        for _ in range(64):
            e = rnd.randint(max(0, ef - 70), ef)
            mant = rnd.getrandbits(52)
            sign = rnd.random() < 0.5
            b = (int(sign) << 63) | (e << 52) | mant
            xs.append(struct.unpack("<d", struct.pack("<Q", b))[0])
        a = bb = cc = 0
        for x in xs:
            v = _fixed_mag(x, ef)
            exact = abs(Fraction(x)) * Fraction(2) ** (1075 - ef)
            fl = math.floor(exact)
            want = fl + 1 if exact - fl >= Fraction(1, 2) else fl
            assert v == want and v < (1 << 53), (x, ef, v, want)
            xh, xl = v >> 27, v & 0x7FFFFFF
            a += xh * xh
            bb += xh * xl
            cc += xl * xl
        assert (a << 54) + (bb << 28) + cc == sum(_fixed_mag(x, ef) ** 2 for x in xs)
        assert a < (1 << 64) and bb < (1 << 64) and cc < (1 << 64)
