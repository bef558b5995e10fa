"""The float64 arg-reduction update of the device code (key compare first,
the special-value path only for candidates; `AccArg<double>` in
xtensor_gb300/csrc/xtg_device.cuh), restated step for step on the host and
checked against the oracle's sequential fold on short sequences rich in
signed zeros, infinities, subnormals and NaNs of every bit pattern that
matters (including the all-ones patterns whose keys equal the empty state's
end keys).  CPU only: this pins the logic; the GPU tests pin the kernels."""
from __future__ import annotations

import struct

import numpy as np

from oracle import oracle as O
from xtensor_gb300.device import HostArray as H

M64 = (1 << 64) - 1
KMIN, KMAX = -(1 << 63), (1 << 63) - 1


def _s64(u):
    return u - (1 << 64) if u >= (1 << 63) else u


def _bits(d):
    return _s64(struct.unpack("<Q", struct.pack("<d", d))[0])


def _unbits(b):
    return struct.unpack("<d", struct.pack("<Q", b & M64))[0]


def _key64(b):
    return b ^ (0x7FFFFFFFFFFFFFFF if b < 0 else 0)


def _special(b):
    hi = (b >> 32) & 0xFFFFFFFF
    return (((hi & 0x7FFFFFFF) - 1) & 0xFFFFFFFF) >= 0x7FEFFFFF


def _isnan_bits(b):
    return (b & 0x7FFFFFFFFFFFFFFF) > 0x7FF0000000000000


def _arg_special(maxop, kv, idx, a, ps):
    b = _bits(a)
    nan = _isnan_bits(b)
    if idx < 0:
        take = (not nan) or ps == 0
    else:
        v = _unbits(_key64(kv))
        take = (a > v) if maxop else (a < v)
    if take:
        return ((KMAX if maxop else KMIN) if nan else _key64(b)), ps
    return kv, idx


def _device_fold(xs, maxop):
    kv, idx = (KMIN if maxop else KMAX), -1
    for ps, a in enumerate(xs):
        b = _bits(a)
        ka = _key64(b)
        if (ka >= kv) if maxop else (ka <= kv):
            if _special(b):
                kv, idx = _arg_special(maxop, kv, idx, a, ps)
                continue
            if ka != kv:
                kv, idx = ka, ps
    return idx


def test_key_first_update_matches_the_fold():
    g = np.random.default_rng(7)
    specials = [0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                _unbits(-1), _unbits(0x7FFFFFFFFFFFFFFF), _unbits(0x7FF0000000000001), _unbits(0xFFF0000000000001)]
    for _ in range(6000):
        n = int(g.integers(1, 12))
        xs = [specials[g.integers(len(specials))] if g.random() < 0.4 else float(g.integers(-3, 4)) for _ in range(n)]
        a = np.array(xs, dtype=np.float64)
        for op, mx in (("argmax", 1), ("argmin", 0)):
            assert _device_fold(xs, mx) == int(O.argreduce(op, H(a), None)), (op, [hex(_bits(v) & M64) for v in xs])


def test_position_free_float64_pass_matches_the_fold_when_it_stands():
    """The position-free first pass of float64 amax / amin (`AccSelFast<double>`):
    the best key and the largest high-word magnitude; when it does not ask
    for the exact pass (no infinity or NaN seen, best key not a zero's),
    its value is the fold's value bit for bit; and it does ask whenever a
    NaN is present."""
    g = np.random.default_rng(8)
    specials = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                -2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308]
    lowest, highest = -1.7976931348623157e308, 1.7976931348623157e308
    asked = 0
    for _ in range(6000):
        n = int(g.integers(1, 12))
        xs = [specials[g.integers(len(specials))] if g.random() < 0.4 else float(g.integers(-3, 4)) * 0.5
              for _ in range(n)]
        a = np.array(xs, dtype=np.float64)
        for op, mx in (("amax", 1), ("amin", 0)):
            kv = _key64(_bits(lowest if mx else highest))
            mh = 0
            for v in xs:
                b = _bits(v)
                mh = max(mh, (b >> 32) & 0x7FFFFFFF)
                ka = _key64(b)
                if (ka >= kv) if mx else (ka <= kv):
                    kv = ka
            exact = mh >= 0x7FF00000 or kv in (0, -1)
            want = O.reduce(op, H(a), None)
            if np.isnan(a).any():
                assert exact
            if exact:
                asked += 1
                continue
            got = _unbits(_key64(kv))
            assert np.array(got).view(np.int64) == np.array(want, np.float64).view(np.int64), (op, xs)
    assert asked < 12000


def test_position_free_float32_pass_matches_the_fold_when_it_stands():
    """The float32 amax / amin position-free pass (`AccSelFast<float>`): one
    NaN-propagating max / min per element (PTX max.NaN / min.NaN); it asks
    for the exact pass when the result is a NaN or a zero, and otherwise its
    value is the fold's, bit for bit."""
    g = np.random.default_rng(9)
    f32 = np.float32
    specials = [f32(0.0), f32(-0.0), f32(np.inf), f32(-np.inf), f32(np.nan), f32(1e-45), f32(-1e-45),
                f32(3.4028235e38), f32(-3.4028235e38)]
    lowest, highest = f32(-3.4028235e38), f32(3.4028235e38)

    def sel_nan(a, b, mx):
        if np.isnan(a) or np.isnan(b):
            return f32(np.nan)
        if a == b:  # +0 / -0: either is fine here, a zero result asks for the exact pass
            return a
        return max(a, b) if mx else min(a, b)

    for _ in range(6000):
        n = int(g.integers(1, 12))
        xs = [specials[g.integers(len(specials))] if g.random() < 0.4 else f32(g.integers(-3, 4) * 0.5)
              for _ in range(n)]
        a = np.array(xs, dtype=np.float32)
        for op, mx in (("amax", 1), ("amin", 0)):
            v = lowest if mx else highest
            for x in xs:
                v = sel_nan(v, x, mx)
            exact = bool(np.isnan(v)) or v == 0
            if np.isnan(a).any():
                assert exact
            if exact:
                continue
            want = O.reduce(op, H(a), None)
            assert np.array(v, np.float32).view(np.int32) == np.array(want, np.float32).view(np.int32), (op, xs)


def test_held_arg_update_equals_the_full_update():
    """Column arg-reductions (`ColStep` with `AccArg<float>`): once a column
    holds a value (idx >= 0) the update is compare-and-select only.  Along
    any chain of positions (a split need not start at position 0) the state
    is the same as with the full update at every element."""
    g = np.random.default_rng(10)
    f32 = np.float32
    vals = [f32(np.nan), f32(np.inf), f32(-np.inf), f32(0.0), f32(-0.0), f32(1.0), f32(-1.0), f32(2.0)]

    def full(state, a, ps, mx):
        v, idx = state
        if idx < 0:
            return (a, ps) if (a == a or ps == 0) else state
        return (a, ps) if ((a > v) if mx else (a < v)) else state

    def held(state, a, ps, mx):
        v, idx = state
        return (a, ps) if ((a > v) if mx else (a < v)) else state

    for _ in range(5000):
        p0 = int(g.integers(0, 3))
        xs = [vals[g.integers(len(vals))] for _ in range(int(g.integers(1, 10)))]
        for mx in (1, 0):
            s_full = s_fast = (f32(0), -1)
            is_held = False
            for k, a in enumerate(xs):
                ps = p0 + k
                s_full = full(s_full, a, ps, mx)
                if is_held:
                    s_fast = held(s_fast, a, ps, mx)
                else:
                    s_fast = full(s_fast, a, ps, mx)
                    is_held = s_fast[1] >= 0
            assert s_full[1] == s_fast[1], (p0, xs, mx)
            assert np.array(s_full[0], np.float32).view(np.int32) == np.array(s_fast[0], np.float32).view(np.int32)
