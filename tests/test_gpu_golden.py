"""The GPU path on the reference's numpy-generated golden vectors
(test/test_extended_xmath_reducers.cpp) and known-answer tests."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu
GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "xmath_reducers.json").read_text())


def test_golden_var_std_gpu():
    g = GOLDEN["var_std"]
    a = DeviceArray.from_numpy(np.array(g["a"], np.float64))
    rtol = 1e-12
    np.testing.assert_allclose(ops.reduce("variance", a).to_numpy(), g["vr_all"], rtol=rtol)
    np.testing.assert_allclose(ops.reduce("variance", a, ddof=1).to_numpy(), g["vr_all_ddof"], rtol=rtol)
    np.testing.assert_allclose(ops.reduce("stddev", a).to_numpy(), g["st_all"], rtol=rtol)
    np.testing.assert_allclose(ops.reduce("variance", a, [0, 2]).to_numpy(), np.array(g["vr"]), rtol=rtol)
    np.testing.assert_allclose(ops.reduce("variance", a, [0, 2], ddof=1).to_numpy(), np.array(g["vr_ddof"]), rtol=rtol)
    np.testing.assert_allclose(ops.reduce("stddev", a, [0, 2]).to_numpy(), np.array(g["st"]), rtol=rtol)
    # the same data in float32: within the float32 tolerance of the fixtures
    a32 = DeviceArray.from_numpy(np.array(g["a"], np.float32))
    np.testing.assert_allclose(ops.reduce("variance", a32, [0, 2]).to_numpy(), np.array(g["vr"]), rtol=2e-6)


def test_golden_weighted_average_gpu():
    g = GOLDEN["average"]
    a = DeviceArray.from_numpy(np.array(g["a"]))
    w = DeviceArray.from_numpy(np.array(g["w"]))
    num = ops.reduce("sum", a * w, [0, 1]).to_numpy()
    den = ops.reduce("sum", w, [0, 1]).to_numpy()
    np.testing.assert_allclose(num / den, np.array(g["av"]), rtol=1e-12)


def test_kat_features_gpu():
    a = np.ones((3, 2, 4, 6, 5))
    for i in range(2):
        for j in range(6):
            a[1, i, 1, j, 1] = 2
    d = DeviceArray.from_numpy(a)
    exp = 12 * np.ones((3, 4, 5))
    exp[1, 1, 1] = 24
    np.testing.assert_array_equal(ops.reduce("sum", d, [1, 3]).to_numpy(), exp)
    assert ops.reduce("sum", d).to_numpy() == 732
    c = DeviceArray.from_numpy(2 * np.ones(34, np.uint8))
    assert ops.reduce("prod", c, acc_dtype="int64").to_numpy() == 1 << 34
    n = DeviceArray.from_numpy(-np.ones(9, np.int32))
    assert ops.reduce("norm_l2", n).to_numpy() == 3.0 and ops.reduce("norm_linf", n).to_numpy() == 1
