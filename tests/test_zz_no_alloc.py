"""The allocation-free float32 sum (xtg_sum_f32_noalloc), called through the
C ABI, against the regular entry point xtg_reduce(sum, all axes).

It serves callers that cannot allocate device memory while they reduce (their
device memory is owned by their own allocator or budget, or they run loops
that must never enter an allocator): its partials live in a static device
array shared by every call.  It runs the same kernels and plan as the regular
entry point, so its result must be bit-identical to xtg_reduce's on the same
input, and within 1e-6 * sum|x| of the FP64 value (the tolerance the sum tests
use).  Calls in a row with different inputs check that whatever the previous
call left in the shared array does not leak into the next result.  The sizes
cover every path of the plan: the empty sum, a single split written directly,
a few splits merged by one thread, and thousands of splits merged by a block.

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
    got = out.to_numpy()
    regular = ops.reduce("sum", dx).to_numpy()
    assert got.tobytes() == regular.tobytes(), (x.size, float(got), float(regular))
    xd = x.astype(np.float64)
    bound = 1e-6 * float(np.abs(xd).sum())
    assert abs(float(got) - float(xd.sum())) <= bound, (x.size, float(got), float(xd.sum()))


def test_noalloc_sum_calls_in_a_row():
    xg.init(0)
    f = _noalloc()
    g = np.random.default_rng(21)

    def lognormal(n):
        return (g.lognormal(0.0, 2.0, n) * g.choice([-1.0, 1.0], n)).astype(np.float32)

    # sign-random lognormal data (heavy cancellation): thousands of splits
    # merged by a block (an odd size: scalar loads), then a size with 16-byte
    # vectors, then a few splits merged by one thread, then one split written
    # directly, then the empty sum, then the first input again
    a = lognormal(1_000_003)
    for x in (a, g.standard_normal(4 << 20).astype(np.float32), lognormal(20_000), lognormal(1_000),
              np.zeros(0, np.float32), a):
        _one_call(f, x)


def test_noalloc_empty_sum_is_zero():
    xg.init(0)
    f = _noalloc()
    out = DeviceArray.from_numpy(np.full((), 7.0, np.float32))
    xg.check(f(None, 0, out.ptr, None))
    assert out.to_numpy().tobytes() == np.float32(0.0).tobytes()


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
