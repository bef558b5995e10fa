"""Parity at the exact benchmark configurations, through the same prebuilt
C-ABI calls bench.py times (bench.GpuStep, bench.C0Step), so the plans that
run here are the plans that earn the numbers: the split counts, bulk-copy
row kernels, column rings and fast selection passes chosen at full size.

C0: A float32 (2048, 2048) U[-1, 1], b float32 (2048,) N(0, 1), seed 0.
  * E = A * b + exp(-A * A): within 4 ulp of the terms' magnitude
    (|A * b| + exp(-A * A)) of the oracle (CUDA's expf vs libm's);
  * r = sum(E, {1}): |r - exact| <= 1e-6 * sum|E| against FP64, and inside
    the reference's own error envelope (|r - ref| <= |ref - exact| +
    1e-6 * sum|E|).
C1: x float32 and float64 (256, 512, 1024) N(0, 1), seed 1.
  * transpose(x, {2, 0, 1}), amax(x, {0, 2}), argmax(x, 1): bit-exact
    against the oracle;
  * (x - mean(x, {2}, kd)) / sqrt(var(x, {2}, kd) + 1e-5): within rel * scale
    of FP64 (rel 4e-6 float32, 1e-12 float64; scale = (|x| + |mean|) /
    sqrt(var + eps)) and inside the reference's envelope around the oracle;
  * a second run of the step gives bit-identical results.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import bench
import xtensor_gb300 as xg
from xtensor_gb300._ffi import check
from xtensor_gb300.device import HostArray
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F32_EPS = 2.0**-24


def _stream():
    st = C.c_void_p()
    check(xg.lib().xtg_stream_create(C.byref(st)))
    return st.value


@pytest.fixture(scope="module")
def c1_run():
    xg.init(0)
    x32, x64 = bench.make_inputs()
    s = _stream()
    step = bench.GpuStep(x32, x64, s)
    step.run()
    check(xg.lib().xtg_stream_sync(s))
    first = [[o.to_numpy() for o in outs] for outs in step.dev_out]
    step.run()
    check(xg.lib().xtg_stream_sync(s))
    second = [[o.to_numpy() for o in outs] for outs in step.dev_out]
    del step
    yield {4: (x32, first[0], second[0]), 8: (x64, first[1], second[1])}


@pytest.mark.parametrize("size", [4, 8], ids=["float32", "float64"])
def test_c1_deterministic(c1_run, size):
    _, a, b = c1_run[size]
    for u, v in zip(a, b):
        assert u.tobytes() == v.tobytes()


@pytest.mark.parametrize("size", [4, 8], ids=["float32", "float64"])
def test_c1_transpose_bit_exact(c1_run, size):
    x, (t, _, _, _), _ = c1_run[size]
    ref = O.assign(HostArray(x.transpose(2, 0, 1)))
    assert t.shape == ref.shape
    assert t.tobytes() == ref.tobytes()


@pytest.mark.parametrize("size", [4, 8], ids=["float32", "float64"])
def test_c1_amax_bit_exact(c1_run, size):
    x, (_, _, am, _), _ = c1_run[size]
    ref = O.reduce("amax", HostArray(x), [0, 2])
    assert am.tobytes() == ref.astype(x.dtype).tobytes()


@pytest.mark.parametrize("size", [4, 8], ids=["float32", "float64"])
def test_c1_argmax_bit_exact(c1_run, size):
    x, (_, _, _, ai), _ = c1_run[size]
    ref = O.argreduce("argmax", HostArray(x), 1)
    np.testing.assert_array_equal(ai.astype(np.int64), ref)


@pytest.mark.parametrize("size", [4, 8], ids=["float32", "float64"])
def test_c1_normalize_within_envelope(c1_run, size):
    x, (_, y, _, _), _ = c1_run[size]
    rel = 4e-6 if size == 4 else 1e-12
    dt = x.dtype
    for i in range(0, x.shape[0], 32):
        xs = x[i:i + 32]
        h = HostArray(xs)
        ref = O.assign((h - xg.rmean(h)) / xg.sqrt(xg.rvar(h) + 1e-5), dtype=dt).astype(np.float64)
        xd = xs.astype(np.float64)
        m = xd.mean(-1, keepdims=True)
        sd = np.sqrt(xd.var(-1, keepdims=True) + 1e-5)
        exact = (xd - m) / sd
        scale = (np.abs(xd) + np.abs(m)) / sd
        got = y[i:i + 32].astype(np.float64)
        err = np.abs(got - exact)
        assert (err <= rel * scale).all(), f"rows {i}..: max err/scale {float(np.max(err / scale))} > {rel}"
        env = np.abs(ref - exact) + rel * scale
        assert (np.abs(got - ref) <= env).all(), f"rows {i}..: outside the reference envelope"


def test_c0_exact_config():
    xg.init(0)
    A, b = bench.make_c0_inputs()
    s = _stream()
    step = bench.C0Step(A, b)
    step.launch(s)
    check(xg.lib().xtg_stream_sync(s))
    E, r = (o.to_numpy() for o in step.dev_out)
    hA, hb = HostArray(A), HostArray(b)
    ref_E = O.assign(hA * hb + xg.exp(-hA * hA))
    Ad = A.astype(np.float64)
    scale = np.abs(Ad * b) + np.exp(-Ad * Ad)
    err = np.abs(E.astype(np.float64) - ref_E)
    assert (err <= 4 * F32_EPS * scale).all(), float(np.max(err / scale))
    ref_r = O.reduce("sum", HostArray(ref_E), [1]).astype(np.float64)
    Ex = E.astype(np.float64)
    exact = Ex.sum(1)
    sa = np.abs(Ex).sum(1)
    got = r.astype(np.float64)
    assert (np.abs(got - exact) <= 1e-6 * sa).all(), float(np.max(np.abs(got - exact) / sa))
    # the reference's own error envelope around its sequential float fold
    exact_ref = ref_E.astype(np.float64).sum(1)
    env = np.abs(ref_r - exact_ref) + 1e-6 * sa + np.abs(exact - exact_ref)
    assert (np.abs(got - ref_r) <= env).all()
