"""Precision configuration at full size: 2^28 elements.

float32 and bfloat16 arrays of sign-random lognormal(mu=0, sigma=2) values
(magnitudes ~1e-6..1e6, heavy cancellation: sum|x| / |sum x| ~ 1e3), seed 2,
reduced with compensated FP32 accumulation; every result's error is stated
against an FP64 evaluation of the same (rounded) data.  int32 U[-2^20, 2^20]
summed into int64 must be bit-exact.

Tolerance: relative error <= 1e-6 against the FP64 value for sum, mean,
variance and norm_l2 (for sum/mean the bound is also checked against
1e-6 * sum|x|, the conditioning-free form).
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray

from util import bf16_bits_to_f32, f32_to_bf16_bits

pytestmark = pytest.mark.gpu
N = 1 << 28


@pytest.fixture(scope="module")
def lognormal():
    g = np.random.default_rng(2)
    mag = g.lognormal(0.0, 2.0, N).astype(np.float32)
    sign = g.integers(0, 2, N, dtype=np.int8) * 2 - 1
    return mag * sign.astype(np.float32)


def _check(dx, x64, what):
    s_exact = float(np.sum(x64))
    abs_sum = float(np.sum(np.abs(x64)))
    n = x64.size
    s = float(ops.reduce("sum", dx).to_numpy())
    m = float(ops.reduce("mean", dx).to_numpy())
    v = float(ops.reduce("variance", dx).to_numpy())
    nl2 = float(ops.reduce("norm_l2", dx).to_numpy())
    mean_exact = s_exact / n
    var_exact = float(np.mean((x64 - mean_exact) ** 2))
    nl2_exact = float(np.sqrt(np.sum(x64 * x64)))
    errs = {
        "sum_rel": abs(s - s_exact) / abs(s_exact),
        "sum_vs_abs": abs(s - s_exact) / abs_sum,
        "mean_rel": abs(m - mean_exact) / abs(mean_exact),
        "var_rel": abs(v - var_exact) / var_exact,
        "norm_l2_rel": abs(nl2 - nl2_exact) / nl2_exact,
    }
    print(what, {k: f"{e:.2e}" for k, e in errs.items()}, "cond", abs_sum / abs(s_exact))
    for k, e in errs.items():
        assert e <= 1e-6, (what, k, e)


def test_float32_lognormal_2e28(lognormal):
    x = lognormal
    dx = DeviceArray.from_numpy(x)
    _check(dx, x.astype(np.float64), "float32")


def test_bfloat16_lognormal_2e28(lognormal):
    bits = f32_to_bf16_bits(lognormal)
    dx = DeviceArray.from_numpy(bits, "bfloat16")
    _check(dx, bf16_bits_to_f32(bits).astype(np.float64), "bfloat16")


def test_int32_to_int64_sum_bit_exact():
    g = np.random.default_rng(2)
    x = g.integers(-(1 << 20), (1 << 20) + 1, N, dtype=np.int32)
    dx = DeviceArray.from_numpy(x)
    got = int(ops.reduce("sum", dx, acc_dtype="int64").to_numpy())
    assert got == int(np.sum(x, dtype=np.int64))
    # the default accumulator is int (wraps like the reference's int sum)
    got32 = int(ops.reduce("sum", dx).to_numpy())
    assert got32 == int(np.sum(x, dtype=np.int64)) - ((int(np.sum(x, dtype=np.int64)) + (1 << 31)) // (1 << 32)) * (1 << 32)


def test_deterministic_repeat(lognormal):
    dx = DeviceArray.from_numpy(lognormal[: 1 << 24])
    a = ops.reduce("sum", dx).to_numpy()
    for _ in range(3):
        assert ops.reduce("sum", dx).to_numpy().tobytes() == a.tobytes()
