"""xtg_assign_reduce: out_e = e, then out_r = reduce(out_e), in one pass of the
row kernel where the plan allows.

The reference evaluates the pair as two statements (`xt::xarray<T> E = e;`
then `xt::sum(E, axes)`: core/xassign.hpp:214-226, reducers/xreducer.hpp:
987-1079).  The fused call must give exactly what the two library calls give
(xtg_assign, then xtg_reduce on the assigned array): E bit for bit, and the
reduction bit for bit — the fused kernel folds the stored values in the
order xtg_reduce folds E (same plan: vector width, splits, groups).  Cases:
C0's expression (one launch, checked through the launched kernel list),
trailing-axis reductions of every kind over 3-D trees, a strided
destination (element stores), a float64 destination of a float32 tree, and
the plans that fall back to the two calls (a column reduction, a destination
that overlaps a leaf, row statistics in the tree).
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu


def _two_calls(e, shape, edt, op, axes, **kw):
    E = DeviceArray.empty(shape, edt)
    xg.assign(E, e)
    r = ops.reduce(op, E, axes=axes, **kw)
    return E.to_numpy(), r.to_numpy()


def _fused(e, E, op, axes, **kw):
    r = ops.assign_reduce(E, e, op, axes=axes, **kw)
    return E.to_numpy(), r.to_numpy()


def test_c0_one_launch_equals_two_calls():
    xg.init(0)
    g = np.random.default_rng(0)
    A = g.uniform(-1, 1, (2048, 2048)).astype(np.float32)
    b = g.standard_normal(2048).astype(np.float32)
    dA, db = DeviceArray.from_numpy(A), DeviceArray.from_numpy(b)
    e = dA * db + xg.exp(-dA * dA)
    E2, r2 = _two_calls(e, A.shape, "float32", "sum", [1])
    E = DeviceArray.empty(A.shape, "float32")
    r = ops.assign_reduce(E, e, "sum", axes=[1])
    kernels = xg.lib().xtg_last_kernels().decode()
    E1, r1 = E.to_numpy(), r.to_numpy()
    assert E1.tobytes() == E2.tobytes()
    assert r1.tobytes() == r2.tobytes()
    names = [k for k in kernels.split(";") if k]
    assert len(names) == 1 and names[0].startswith("k_reduce_row<") and names[0].endswith(", 1, float>"), names


@pytest.mark.parametrize("op,kw", [("sum", {}), ("mean", {}), ("prod", {}), ("amax", {}), ("amin", {}),
                                   ("norm_l2", {}), ("norm_l1", {}), ("variance", {}), ("stddev", {"ddof": 1}),
                                   ("sum", {"keep_dims": True}), ("sum", {"initial": 2.5})])
@pytest.mark.parametrize("axes", [[2], [1, 2]])
def test_trailing_axes_equal_two_calls(op, kw, axes):
    xg.init(0)
    g = np.random.default_rng(7)
    x = g.standard_normal((6, 40, 300)).astype(np.float32)
    y = (g.random((300,)) + 0.5).astype(np.float32)
    dx, dy = DeviceArray.from_numpy(x), DeviceArray.from_numpy(y)
    e = (dx * dy - 0.25) if op != "prod" else (dx * 0.01 + 1)
    E2, r2 = _two_calls(e, x.shape, "float32", op, axes, **kw)
    E = DeviceArray.empty(x.shape, "float32")
    E1, r1 = _fused(e, E, op, axes, **kw)
    assert E1.tobytes() == E2.tobytes()
    assert r1.tobytes() == r2.tobytes(), (op, kw, axes)


def test_strided_destination_and_wider_type():
    xg.init(0)
    g = np.random.default_rng(8)
    x = g.standard_normal((64, 1000)).astype(np.float32)
    dx = DeviceArray.from_numpy(x)
    # every other row of a larger array: not contiguous across rows
    big = DeviceArray.from_numpy(np.zeros((128, 1000), np.float32))
    E = big[::2]
    r1 = ops.assign_reduce(E, dx * 3 + 1, "sum", axes=[1]).to_numpy()
    want_E = x * np.float32(3) + np.float32(1)
    np.testing.assert_array_equal(big.to_numpy()[::2], want_E)
    np.testing.assert_array_equal(big.to_numpy()[1::2], 0)
    _, r2 = _two_calls(dx * 3 + 1, x.shape, "float32", "sum", [1])
    assert r1.tobytes() == r2.tobytes()
    # float64 destination of a float32 tree: the values are converted, then reduced in double
    E64 = DeviceArray.empty(x.shape, "float64")
    r3 = ops.assign_reduce(E64, dx * dx, "sum", axes=[1]).to_numpy()
    E4, r4 = _two_calls(dx * dx, x.shape, "float64", "sum", [1])
    assert E64.to_numpy().tobytes() == E4.tobytes()
    assert r3.tobytes() == r4.tobytes()
    # column-strided destination (element stores along the reduced run)
    big2 = DeviceArray.from_numpy(np.zeros((64, 2000), np.float32))
    E5 = big2[:, ::2]
    r5 = ops.assign_reduce(E5, dx - 2, "amax", axes=[1]).to_numpy()
    np.testing.assert_array_equal(big2.to_numpy()[:, ::2], x - np.float32(2))
    np.testing.assert_array_equal(r5, (x - np.float32(2)).max(1))


def test_fallback_plans_equal_two_calls():
    xg.init(0)
    g = np.random.default_rng(9)
    x = g.standard_normal((300, 512)).astype(np.float32)
    dx = DeviceArray.from_numpy(x)
    # column reduction (reduced axis strided): two calls
    E = DeviceArray.empty(x.shape, "float32")
    r1 = ops.assign_reduce(E, dx * 2, "sum", axes=[0]).to_numpy()
    E2, r2 = _two_calls(dx * 2, x.shape, "float32", "sum", [0])
    assert E.to_numpy().tobytes() == E2.tobytes() and r1.tobytes() == r2.tobytes()
    # destination that is a leaf (in-place update): two calls
    d2 = DeviceArray.from_numpy(x)
    r3 = ops.assign_reduce(d2, d2 * 2, "variance", axes=[1]).to_numpy()
    np.testing.assert_array_equal(d2.to_numpy(), x * np.float32(2))
    r4 = ops.reduce("variance", d2, axes=[1]).to_numpy()
    assert r3.tobytes() == r4.tobytes()
    # row statistics inside the tree: two calls
    E3 = DeviceArray.empty(x.shape, "float32")
    r5 = ops.assign_reduce(E3, dx - xg.rmean(dx), "sum", axes=[1]).to_numpy()
    E6, r6 = _two_calls(dx - xg.rmean(dx), x.shape, "float32", "sum", [1])
    assert E3.to_numpy().tobytes() == E6.tobytes() and r5.tobytes() == r6.tobytes()


def test_errors():
    xg.init(0)
    dx = DeviceArray.from_numpy(np.ones((4, 5), np.float32))
    with pytest.raises(xg.XtgError) as ei:
        ops.assign_reduce(DeviceArray.empty((4, 6), "float32"), dx * 2, "sum", axes=[1])
    assert ei.value.status == 5  # destination shape
    with pytest.raises(xg.XtgError) as ei:
        ops.assign_reduce(DeviceArray.empty((4, 5), "float32"), dx * 2, "sum", axes=[1, 0])
    assert ei.value.status == 3  # unsorted axes
