"""The allocation-free float32 sum (xtg_sum_f32_noalloc), called through the
C ABI, against the regular entry point xtg_reduce(sum, all axes).

It is for callers that cannot allocate device memory while they reduce
(stream capture, a caller-owned memory budget): its partials live in a static
device buffer shared by every call.  Two calls in a row with different inputs
check that whatever the previous call left in that buffer does not leak into
the next result.  Tolerance: the one the sum tests use, 1e-6 * sum|x| against
the regular entry point and against an FP64 evaluation.

This file is collected last so that a run stopping at its first failure has
already run every other test; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu


def _noalloc():
    L = xg.lib()
    f = L.xtg_sum_f32_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    return f


def _one_call(f, x: np.ndarray) -> None:
    dx = DeviceArray.from_numpy(x)
    out = DeviceArray.empty((), "float32")
    xg.check(f(dx.ptr, x.size, out.ptr, None))
    got = float(out.to_numpy())
    regular = float(ops.reduce("sum", dx).to_numpy())
    xd = x.astype(np.float64)
    bound = 1e-6 * float(np.abs(xd).sum())
    assert abs(got - regular) <= bound, (got, regular)
    assert abs(got - float(xd.sum())) <= bound, (got, float(xd.sum()))


def test_noalloc_sum_two_calls():
    xg.init(0)
    f = _noalloc()
    g = np.random.default_rng(21)
    # sign-random lognormal data (heavy cancellation); an odd size (scalar
    # loads, many chunks) then a size with 16-byte vectors.
    a = (g.lognormal(0.0, 2.0, 1_000_003) * g.choice([-1.0, 1.0], 1_000_003)).astype(np.float32)
    b = g.standard_normal(4 << 20).astype(np.float32)
    _one_call(f, a)
    _one_call(f, b)


def test_noalloc_rejects_oversized_plan():
    xg.init(0)
    f = _noalloc()
    x = DeviceArray.from_numpy(np.ones(1 << 22, np.float32))
    out = DeviceArray.empty((), "float32")
    xg.set_option("reduce.target_items", 1 << 20)
    xg.set_option("reduce.min_chunk", 1)
    try:
        st = f(x.ptr, 1 << 22, out.ptr, None)
        assert st == 9, st  # XTG_ERR_UNSUPPORTED, before any launch
        assert b"static" in xg.lib().xtg_last_error()
    finally:
        xg.set_option("reduce.target_items", -1)
        xg.set_option("reduce.min_chunk", -1)
    xg.check(f(x.ptr, 1 << 22, out.ptr, None))
    assert float(out.to_numpy()) == float(1 << 22)
