"""xtg_reduce_moments: sum, mean, variance and norm_l2 from one pass.

The reference computes each statistic with its own reducer call
(core/xmath.hpp:367-423 sum, 1828-1911 mean, 2082-2103 variance;
reducers/xnorm.hpp:494-526 norm_l2).  When the plan streams (a full
reduction of one contiguous float32 / bfloat16 array), the library reads the
input once and keeps the four reducers' accumulators side by side, each fed
what its own kernel feeds it: every result must equal the corresponding
xtg_reduce call bit for bit.  Other plans run the four reductions in turn
(trivially equal).  The one-pass form must launch the streaming kernel once.
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import check, last_kernels
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu

SIZES = [(1 << 26) + 4000, 3 << 24, 1 << 22]


def data(n, dt, seed=141):
    g = np.random.default_rng(seed)
    x = (g.lognormal(0.0, 2.0, n) * np.where(g.random(n) < 0.5, -1.0, 1.0) + 3.0).astype(np.float32)
    if dt == "bfloat16":
        from util import f32_to_bf16_bits
        x = f32_to_bf16_bits(x)
    return DeviceArray.from_numpy(x, dt)


def separate(d, ddof=0, **kw):
    return {nm: ops.reduce(nm, d, ddof=ddof if nm == "variance" else 0, **kw).to_numpy() for nm in ops.MOMENTS}


@pytest.mark.parametrize("cta_chunk", [None, 64])
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dt", ["float32", "bfloat16"])
def test_one_pass_equals_separate_calls(n, dt, cta_chunk):
    xg.init(0)
    d = data(n, dt)
    if cta_chunk is not None:
        xg.set_option("reduce.cta_chunk", cta_chunk)
    try:
        for ddof in (0, 1):
            got = ops.reduce_moments(d, ddof=ddof)
            ks = last_kernels()
            want = separate(d, ddof=ddof)
            if cta_chunk is not None or n >= (1 << 25):
                assert [k.split("<")[0] for k in ks][0] == "k_reduce_stream", ks
                assert len([k for k in ks if k.startswith("k_reduce_stream")]) == 1, ks
            for nm in ops.MOMENTS:
                a, b = got[nm].to_numpy(), want[nm]
                assert a.dtype == b.dtype and a.shape == b.shape
                assert a.tobytes() == b.tobytes(), (nm, ddof, a, b)
    finally:
        xg.set_option("reduce.cta_chunk", -1)
    check(xg.lib().xtg_check_device_errors())


@pytest.mark.parametrize("which", [("variance",), ("mean", "norm_l2"), ("sum",), ("norm_l2", "variance", "sum")])
def test_subsets_of_outputs(which):
    xg.init(0)
    d = data(3 << 24, "float32", seed=142)
    got = ops.reduce_moments(d, which=which)
    assert set(got) == set(which)
    want = separate(d)
    for nm in which:
        assert got[nm].to_numpy().tobytes() == want[nm].tobytes(), nm


@pytest.mark.parametrize("case", ["axis", "float64", "int32", "expression", "strided"])
def test_other_plans_run_the_four_reductions(case):
    xg.init(0)
    g = np.random.default_rng(143)
    kw = {}
    if case == "axis":
        d = DeviceArray.from_numpy(g.standard_normal((64, 4096)).astype(np.float32))
        kw = {"axes": [1]}
    elif case == "float64":
        d = DeviceArray.from_numpy(g.standard_normal(1 << 22))
    elif case == "int32":
        d = DeviceArray.from_numpy(g.integers(-1000, 1000, 1 << 22).astype(np.int32))
    elif case == "expression":
        d = DeviceArray.from_numpy(g.standard_normal(1 << 22).astype(np.float32)) * 2.0 + 1.0
    else:
        d = DeviceArray.from_numpy(g.standard_normal(1 << 23).astype(np.float32))[::2]
    got = ops.reduce_moments(d, **kw)
    want = separate(d, **kw)
    for nm in ops.MOMENTS:
        assert got[nm].to_numpy().tobytes() == want[nm].tobytes(), (case, nm)


def test_errors():
    xg.init(0)
    d = DeviceArray.from_numpy(np.ones(1 << 20, np.float32))
    with pytest.raises(ValueError):
        ops.reduce_moments(d, which=("median",))
    ex, keep = __import__("xtensor_gb300.expr", fromlist=["lower"]).lower(d)
    rd = ops.make_desc("sum")
    import ctypes as C
    # no destination at all
    assert xg.lib().xtg_reduce_moments(C.byref(ex), C.byref(rd), None, None, None, None, None) == 1
    # a destination of the wrong type
    bad = DeviceArray.empty((), "float32").xtg_array()
    with pytest.raises(xg.XtgError):
        check(xg.lib().xtg_reduce_moments(C.byref(ex), C.byref(rd), None, C.byref(bad), None, None, None))
