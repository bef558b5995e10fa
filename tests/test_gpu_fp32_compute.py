"""float64 scalars in float32 trees: the fp32_compute option (on by default).

C++ promotion makes `x * 0.1` on float32 x a double expression: the reference
multiplies in double and rounds once, when it stores into the float32
container (include/xtensor/core/xoperation.hpp:30-143 for the result types,
core/xassign.hpp:613-642 for the final conversion).  With fp32_compute on,
the library evaluates such nodes in float32 (GB300's FP64 rate is a small
fraction of its FP32 rate): each float64 scalar is rounded to float32 once
and every operation rounds to float32.

Stated bound, checked here against the oracle's double-promoting evaluation
on literals that float32 cannot represent (0.1, 1e-5, 0.3, 1.7, 3.3, ...):
for a tree of k arithmetic nodes,

    |gpu - ref| <= (2k + 1) * 2^-24 * S,

where S is the same tree evaluated in FP64 on the magnitudes of its leaves
and scalars with every subtraction turned into an addition (the standard
forward-error bound of k float32 roundings, k scalar roundings and the
reference's own final rounding).  With fp32_compute off the library follows
C++ promotion and matches the oracle bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300.device import DeviceArray, HostArray
from oracle import oracle as O

pytestmark = pytest.mark.gpu

U = 2.0**-24

# (tree over (x, y), k arithmetic nodes, magnitude tree over (|x|, |y|) in FP64)
TREES = [
    (lambda x, y: x * 0.1, 1, lambda x, y: x * 0.1),
    (lambda x, y: x * 0.1 + 1e-5, 2, lambda x, y: x * 0.1 + 1e-5),
    (lambda x, y: (x - 0.3) * 1.7 + y * 0.2, 4, lambda x, y: (x + 0.3) * 1.7 + y * 0.2),
    (lambda x, y: x / 3.3 - 0.01, 2, lambda x, y: x / 3.3 + 0.01),
    (lambda x, y: x * x * 0.7 - y * 1e-3 + 2.2, 5, lambda x, y: x * x * 0.7 + y * 1e-3 + 2.2),
]


@pytest.fixture(scope="module")
def data():
    xg.init(0)
    g = np.random.default_rng(31)
    x = g.standard_normal((37, 1024)).astype(np.float32)
    y = (g.standard_normal((1024,)) * 10).astype(np.float32)
    x[0, :8] = [0.0, -0.0, 1e-30, -1e-30, 3e4, -3e4, 0.3, 1e-4]
    return x, y


@pytest.mark.parametrize("i", range(len(TREES)))
def test_fp32_compute_within_stated_bound(data, i):
    f, k, mag = TREES[i]
    x, y = data
    dx, dy = DeviceArray.from_numpy(x), DeviceArray.from_numpy(y)
    out = DeviceArray.empty(x.shape, "float32")
    xg.assign(out, f(dx, dy))
    got = out.to_numpy().astype(np.float64)
    ref = O.assign(f(HostArray(x), HostArray(y)), dtype="float32").astype(np.float64)
    S = mag(np.abs(x.astype(np.float64)), np.abs(y.astype(np.float64)))
    err = np.abs(got - ref)
    bound = (2 * k + 1) * U * S
    assert (err <= bound).all(), f"tree {i}: max err / (U*S) = {float(np.max(err / (U * S)))} > {2 * k + 1}"


@pytest.mark.parametrize("i", range(len(TREES)))
def test_fp32_compute_off_follows_cpp_promotion(data, i):
    f, _, _ = TREES[i]
    x, y = data
    dx, dy = DeviceArray.from_numpy(x), DeviceArray.from_numpy(y)
    out = DeviceArray.empty(x.shape, "float32")
    xg.set_option("fp32_compute", 0)
    try:
        xg.assign(out, f(dx, dy))
    finally:
        xg.set_option("fp32_compute", -1)
    ref = O.assign(f(HostArray(x), HostArray(y)), dtype="float32")
    assert out.to_numpy().tobytes() == ref.tobytes()


def test_c1_literal_in_row_normalisation(data):
    """C1's `+ 1e-5` inside the fused row tree on float32 data: within the
    normalisation tolerance of the FP64 value (4e-6 of (|x| + |mean|) /
    sqrt(var + eps)), which the demoted evaluation must keep."""
    x, _ = data
    dx = DeviceArray.from_numpy(x)
    out = DeviceArray.empty(x.shape, "float32")
    xg.assign(out, (dx - xg.rmean(dx)) / xg.sqrt(xg.rvar(dx) + 1e-5))
    xd = x.astype(np.float64)
    m = xd.mean(-1, keepdims=True)
    sd = np.sqrt(xd.var(-1, keepdims=True) + 1e-5)
    scale = (np.abs(xd) + np.abs(m)) / sd
    assert (np.abs(out.to_numpy() - (xd - m) / sd) <= 4e-6 * scale).all()
