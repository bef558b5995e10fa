"""GPU reads and writes through index_view / filter / filtration /
masked_view against the oracle and the reference's view tests.  Every
result here is bit-exact (elementwise arithmetic in the same C++ types)."""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import XtgError, last_kernels
from xtensor_gb300.device import DeviceArray, HostArray as H
from oracle import oracle as O

from util import rng

pytestmark = pytest.mark.gpu


def dev(a, dtype=None):
    return DeviceArray.from_numpy(a, dtype)


def test_reference_index_view_kats():
    e = np.arange(9, dtype=np.float64).reshape(3, 3) / 7.0
    d = dev(e)
    idx = [[1, 1], [1, 2], [2, 2]]
    np.testing.assert_array_equal(ops.index_view(d, idx).to_numpy(), [e[1, 1], e[1, 2], e[2, 2]])
    ops.index_assign(d, idx, 3.0, "+=")
    assert d.to_numpy()[1, 1] == e[1, 1] + 3
    ops.index_assign(d, idx, 123.0)
    h = d.to_numpy()
    assert h[1, 1] == h[1, 2] == h[2, 2] == 123
    ops.index_assign(d, idx, dev(np.array([3.0, 3.0, 3.0])))
    assert d.to_numpy()[2, 2] == 3
    # index view over an expression (indices_on_function :112-129)
    fn = d * 3 - 120
    got = ops.index_view(fn, idx).to_numpy()
    np.testing.assert_array_equal(got, O.index_view(H(d.to_numpy()) * 3 - 120, idx))


def test_reference_filter_kats():
    e = np.eye(3)
    d = dev(e)
    assert ops.filter(d, d > 0).to_numpy()[0] == 1
    ops.filter_assign(d, d > 0, 2.0, "+=")
    assert d.to_numpy()[1, 1] == 3
    ops.filter_assign(d, d > 0, dev(np.array([1.0, 2.0, 3.0])), "+=")
    h = d.to_numpy()
    assert h[1, 1] == 5 and h[2, 2] == 6
    f = dev(np.eye(3))
    ops.filter_assign(f, f < 1, 2.0)
    np.testing.assert_array_equal(f.to_numpy(), [[1, 2, 2], [2, 1, 2], [2, 2, 1]])
    a = dev(np.array([[1.0, 5, 3], [4, 5, 6]]))
    ops.filter_assign(a, a >= 5, 2.0, "+=")
    np.testing.assert_array_equal(a.to_numpy(), [[1, 7, 3], [4, 7, 8]])
    a = dev(np.array([[1.0, 5, 3], [4, 5, 6]]))
    b = dev(np.array([[1.0, 5, 3], [4, 5, 6]]))
    ops.filter_assign(a, a > 3, ops.filter(b, b > 3), "+=")
    np.testing.assert_array_equal(a.to_numpy(), [[1, 10, 3], [8, 10, 12]])
    x = dev(np.array([[[1, 3], [2, 4]], [[5, 7], [6, 8]]], np.int32))
    c = dev(np.array([[[True, True], [False, False]], [[True, True], [False, False]]]))
    np.testing.assert_array_equal(ops.filter(x, c).to_numpy(), [1, 3, 5, 7])


def test_reference_masked_view_kats():
    data = dev(np.array([[1.0, -2, 3], [4, 5, -6], [7, 8, -9]]))
    mask = dev(np.array([[True, True, True], [True, False, False], [True, False, True]]))
    ops.masked_assign(data, mask, 3.65)
    np.testing.assert_array_equal(data.to_numpy(), [[3.65, 3.65, 3.65], [3.65, 5, -6], [3.65, 8, 3.65]])
    ops.masked_assign(data, mask, 3.0, "+=")
    np.testing.assert_array_equal(data.to_numpy(), [[6.65, 6.65, 6.65], [6.65, 5, -6], [6.65, 8, 6.65]])
    data = dev(np.array([[1.0, -2, 3], [4, 5, -6], [7, 8, -9]]))
    data2 = dev(np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6], [0.7, 0.8, 0.9]]))
    ops.masked_assign(data, mask, data2)
    np.testing.assert_array_equal(data.to_numpy(), [[0.1, 0.2, 0.3], [0.4, 5, -6], [0.7, 8, 0.9]])
    d = dev(np.array([[0, 1], [2, 3], [4, 5]], np.uint64))
    ops.masked_assign(d[0], dev(np.array([False, True])), 10, "+=")
    h = d.to_numpy()
    assert h[0, 0] == 0 and h[0, 1] == 11


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64"])
@pytest.mark.parametrize("op", ["=", "+=", "-=", "*=", "/="])
def test_parity_random(dt, op):
    g = rng(40)
    shape = (33, 47, 9)
    if dt.startswith("float"):
        a = g.standard_normal(shape).astype(dt)
        s = g.standard_normal(shape).astype(dt)
    else:
        a = g.integers(-20, 20, shape).astype(dt)
        s = g.integers(1, 9, shape).astype(dt)
    # masked assignment with a broadcast mask and an expression source
    m = g.random((1, 47, 9)) < 0.4
    d = dev(a)
    ops.masked_assign(d, dev(m), dev(s) * 2 + 1, op)
    np.testing.assert_array_equal(d.to_numpy(), O.masked_assign(a.copy(), H(m), H(s) * 2 + 1, op))
    # filter reads and writes
    cond_h = H(a) > (0 if dt.startswith("float") else 3)
    cond_d = dev(a) > (0 if dt.startswith("float") else 3)
    np.testing.assert_array_equal(ops.filter(dev(a) * 3, cond_d).to_numpy(), O.filter(H(a) * 3, cond_h))
    cnt = ops.filter_count(cond_d)
    src = s.reshape(-1)[:cnt].copy()
    d = dev(a)
    ops.filter_assign(d, dev(a) > (0 if dt.startswith("float") else 3), dev(src), op)
    np.testing.assert_array_equal(d.to_numpy(), O.filter_assign(a.copy(), cond_h, H(src), op))
    # index views: unique coordinates
    flat = g.choice(a.size, 500, replace=False)
    idx = np.stack(np.unravel_index(flat, shape), 1)
    np.testing.assert_array_equal(ops.index_view(dev(a), idx).to_numpy(), O.index_view(H(a), idx))
    d = dev(a)
    vals = s.reshape(-1)[:500].copy()
    ops.index_assign(d, idx, dev(vals), op)
    np.testing.assert_array_equal(d.to_numpy(), O.index_assign(a.copy(), idx, H(vals), op))


def test_assignment_through_aliasing_views():
    """a = transpose(a) and a masked write of a transposed a evaluate through
    a temporary (as the reference's `=` does), not in place."""
    g = rng(41)
    a = g.standard_normal((64, 64)).astype(np.float32)
    d = dev(a)
    xg.assign(d, d.transpose((1, 0)))
    np.testing.assert_array_equal(d.to_numpy(), a.T)
    d = dev(a)
    m = g.random((64, 64)) < 0.5
    ops.masked_assign(d, dev(m), d.transpose((1, 0)) + 1)
    np.testing.assert_array_equal(d.to_numpy(), np.where(m, a.T + 1, a))
    # shifted overlap: d[1:] = d[:-1]
    d = dev(a)
    xg.assign(d[1:], d[:-1])
    np.testing.assert_array_equal(d.to_numpy()[1:], a[:-1])


def test_out_of_range_coordinates_are_skipped_and_reported():
    x = dev(np.arange(12, dtype=np.float64).reshape(3, 4))
    out = ops.index_view(x, [[0, 0], [3, 1], [2, 3]])  # (3, 1) is outside
    got = out.to_numpy()
    assert got[0] == 0 and got[2] == 11
    from xtensor_gb300._ffi import check
    with pytest.raises(XtgError) as ei:
        check(xg.lib().xtg_check_device_errors())
    assert ei.value.status == 4
    check(xg.lib().xtg_check_device_errors())  # cleared


def test_errors():
    d = dev(np.ones((3, 4)))
    with pytest.raises(XtgError):
        ops.filter(d, dev(np.ones((4,), bool)))  # condition shape must equal e's
    with pytest.raises(XtgError):
        ops.filter_assign(d, d > 0, dev(np.ones(5)))  # 12 selected, 5 values
