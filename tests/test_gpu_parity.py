"""GPU parity: every kernel family against the oracle on seeded inputs.

Tolerances (stated here, checked below):
  * integer, bool and index results, copies and transposes: bit-exact;
  * float32/float64 trees of + - * / sqrt, comparisons, select: bit-exact
    (IEEE operations in the same order, no fused multiply-add);
  * trees with exp/log/sin/cos/tanh: <= 4 ulp of the magnitude of the terms
    (CUDA's single-precision exp is within 2 ulp, the reference's libm within 1);
  * float32 sums/means/norms: |gpu - exact| <= 1e-6 * sum|x| against an FP64
    evaluation, and within the reference's own error envelope
    (|gpu - ref| <= |ref - exact| + 1e-6 * sum|x|);
  * variance/stddev: relative 1e-6 (float32 data) / 1e-12 (float64 data) of
    the FP64 value;
  * amax/amin: bit-exact.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray, HostArray
from oracle import oracle as O

from util import assert_close_rel, assert_ulp, bf16_bits_to_f32, f32_to_bf16_bits, rng

pytestmark = pytest.mark.gpu

F32_EPS = 2.0**-24


def dev(a, dtype=None):
    return DeviceArray.from_numpy(a, dtype)


def H(a, dtype=None):
    return HostArray(a, dtype)


# ---------------------------------------------------------------------------- assign
def test_c0_expression_small():
    g = rng(0)
    A = g.uniform(-1, 1, (64, 96)).astype(np.float32)
    b = g.standard_normal(96).astype(np.float32)
    dA, db = dev(A), dev(b)
    out = DeviceArray.empty(A.shape, "float32")
    xg.assign(out, dA * db + xg.exp(-dA * dA))
    got = out.to_numpy()
    ref = O.assign(H(A) * H(b) + xg.exp(-H(A) * H(A)))
    scale = np.abs(A * b) + np.exp(-(A.astype(np.float64) ** 2))
    assert_close_rel(got, ref, 4 * F32_EPS, scale, "A*b + exp(-A*A)")


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64", "uint8", "int16"])
def test_arith_bit_exact(dt):
    g = rng(1)
    if dt.startswith("float"):
        a = g.standard_normal((17, 33)).astype(dt)
        b = g.standard_normal((33,)).astype(dt) + 2
    else:
        info = np.iinfo(dt)
        a = g.integers(max(info.min, -1000), min(info.max, 1000), (17, 33)).astype(dt)
        b = g.integers(1, min(info.max, 100), (33,)).astype(dt)
    for f in [lambda x, y: x + y, lambda x, y: x - y * y, lambda x, y: x * y - x,
              lambda x, y: xg.maximum(x, y) - xg.minimum(x, y), lambda x, y: xg.where(x > y, x, y * 2)]:
        e_d = f(dev(a), dev(b))
        e_h = f(H(a), H(b))
        code = O.expr_dtype(e_h)
        assert xg.expr_dtype(e_d) == code
        out = DeviceArray.empty(a.shape, code)
        xg.assign(out, e_d)
        ref = O.assign(e_h)
        np.testing.assert_array_equal(out.to_numpy(), ref)


def test_division_and_sqrt_bit_exact():
    g = rng(2)
    a = g.standard_normal((50, 70)).astype(np.float32)
    b = (g.random((70,)) + 0.5).astype(np.float32)
    out = DeviceArray.empty(a.shape, "float32")
    xg.assign(out, xg.sqrt(xg.abs_(dev(a))) / dev(b))
    ref = O.assign(xg.sqrt(xg.abs_(H(a))) / H(b))
    assert_ulp(out.to_numpy(), ref, 0, "sqrt/div")


def test_mixed_type_promotion():
    g = rng(3)
    a = g.integers(-50, 50, (8, 9)).astype(np.int32)
    b = g.standard_normal((9,)).astype(np.float64)
    c = g.integers(0, 200, (8, 1)).astype(np.uint8)
    e_d = dev(a) * dev(b) + dev(c)
    e_h = H(a) * H(b) + H(c)
    assert O.expr_dtype(e_h) == xg.DTYPES["float64"] == xg.expr_dtype(e_d)
    out = DeviceArray.empty((8, 9), "float64")
    xg.assign(out, e_d)
    np.testing.assert_array_equal(out.to_numpy(), O.assign(e_h))
    # uint8 + uint8 is int in C++: no wrap
    u = g.integers(0, 256, (40,)).astype(np.uint8)
    e = dev(u) + dev(u)
    assert xg.expr_dtype(e) == xg.DTYPES["int32"]
    o2 = DeviceArray.empty((40,), "int32")
    xg.assign(o2, e)
    np.testing.assert_array_equal(o2.to_numpy(), u.astype(np.int32) * 2)
    # storing into uint8 wraps like a static_cast
    o3 = DeviceArray.empty((40,), "uint8")
    xg.assign(o3, e)
    np.testing.assert_array_equal(o3.to_numpy(), (u.astype(np.int32) * 2).astype(np.uint8))


def test_scalars_and_literals():
    g = rng(4)
    a = g.standard_normal((10, 11)).astype(np.float32)
    # 2.0 is a double literal: a * 2.0 is exact in float, the tree is float64 in C++
    for f in [lambda x: x * 2.0 + 1, lambda x: 3 - x, lambda x: x / np.float32(4.0), lambda x: -x + np.float32(0.5)]:
        out = DeviceArray.empty(a.shape, "float32")
        xg.assign(out, f(dev(a)))
        ref = O.assign(f(H(a)), dtype="float32")
        assert_ulp(out.to_numpy(), ref, 0, "scalar")


def test_broadcast_shapes_and_errors():
    g = rng(5)
    a = g.standard_normal((3, 1, 5)).astype(np.float32)
    b = g.standard_normal((4, 1)).astype(np.float32)
    e = dev(a) + dev(b)
    assert xg.broadcast_shape(e) == (3, 4, 5)
    out = DeviceArray.empty((3, 4, 5), "float32")
    xg.assign(out, e)
    np.testing.assert_array_equal(out.to_numpy(), a + b)
    with pytest.raises(xg.XtgError) as ei:
        xg.broadcast_shape(dev(np.zeros((3, 4), np.float32)) + dev(np.zeros((5,), np.float32)))
    assert ei.value.status == 2  # broadcast_error
    # destination of the wrong shape
    with pytest.raises(xg.XtgError):
        xg.assign(DeviceArray.empty((3, 4), "float32"), e)


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int8", "bfloat16"])
@pytest.mark.parametrize("perm", list(itertools.permutations(range(3))))
def test_transpose_bit_exact(dt, perm):
    g = rng(6)
    shape = (37, 70, 45)
    if dt == "bfloat16":
        x = f32_to_bf16_bits(g.standard_normal(shape).astype(np.float32))
    elif dt.startswith("float"):
        x = g.standard_normal(shape).astype(dt)
    else:
        x = g.integers(-100, 100, shape).astype(dt)
    d = dev(x, dt)
    t = d.transpose(perm)
    out = DeviceArray.empty(t.shape, dt)
    xg.assign(out, t)
    np.testing.assert_array_equal(out.to_numpy(), np.ascontiguousarray(x.transpose(perm)))


@pytest.mark.parametrize("dt", ["float32", "float64", "int8", "bfloat16"])
@pytest.mark.parametrize("perm", [(0, 2, 1), (2, 0, 1), (1, 2, 0), (2, 1, 0)])
def test_transpose_interior_and_edge_tiles(dt, perm):
    """Shapes with whole 64x64 (and 32x32) tiles plus ragged edges, so both
    the unchecked interior path and the bounds-checked edge path run."""
    g = rng(16)
    shape = (3, 129, 257)
    if dt == "bfloat16":
        x = f32_to_bf16_bits(g.standard_normal(shape).astype(np.float32))
    elif dt.startswith("float"):
        x = g.standard_normal(shape).astype(dt)
    else:
        x = g.integers(-100, 100, shape).astype(dt)
    d = dev(x, dt)
    out = DeviceArray.empty(d.transpose(perm).shape, dt)
    xg.assign(out, d.transpose(perm))
    np.testing.assert_array_equal(out.to_numpy(), np.ascontiguousarray(x.transpose(perm)))


def test_transpose_with_elementwise_and_views():
    g = rng(7)
    x = g.standard_normal((64, 48)).astype(np.float32)
    y = g.standard_normal((48,)).astype(np.float32)
    dx, dy = dev(x), dev(y)
    out = DeviceArray.empty((48, 64), "float32")
    xg.assign(out, dx.transpose() * np.float32(2))
    np.testing.assert_array_equal(out.to_numpy(), x.T * np.float32(2))
    # strided views (steps, negative steps, offsets)
    v = dx[1::3, ::-2]
    o2 = DeviceArray.empty(v.shape, "float32")
    xg.assign(o2, v + np.float32(1))
    np.testing.assert_array_equal(o2.to_numpy(), x[1::3, ::-2] + np.float32(1))
    # assignment into a strided destination view
    big = DeviceArray.from_numpy(np.zeros((64, 48), np.float32))
    dst = big[::2, 3:43]
    xg.assign(dst, dx[::2, 3:43] * dx[::2, 3:43])
    exp_ = np.zeros((64, 48), np.float32)
    exp_[::2, 3:43] = x[::2, 3:43] * x[::2, 3:43]
    np.testing.assert_array_equal(big.to_numpy(), exp_)


def test_unaligned_and_odd_sizes():
    g = rng(8)
    for n in [1, 3, 5, 31, 33, 1023, 4097]:
        a = g.standard_normal(n + 1).astype(np.float32)
        d = dev(a)[1:]  # 4-byte offset: no 16-byte vectors
        out = DeviceArray.empty((n,), "float32")
        xg.assign(out, d * d + np.float32(1))
        np.testing.assert_array_equal(out.to_numpy(), a[1:] * a[1:] + np.float32(1))


def test_math_functions_ulp():
    g = rng(9)
    x = g.uniform(0.1, 4, (300,)).astype(np.float32)
    for fn, name in [(xg.exp, "exp"), (xg.log, "log"), (xg.sin, "sin"), (xg.cos, "cos"), (xg.tanh, "tanh")]:
        out = DeviceArray.empty(x.shape, "float32")
        xg.assign(out, fn(dev(x)))
        ref = O.assign(fn(H(x)))
        assert_ulp(out.to_numpy(), ref, 4, name)
    xd = x.astype(np.float64)
    out = DeviceArray.empty(x.shape, "float64")
    xg.assign(out, xg.exp(dev(xd)))
    assert_ulp(out.to_numpy(), O.assign(xg.exp(H(xd))), 2, "exp f64")


# ------------------------------------------------------------------------------- reductions
SHAPES_AXES = [
    ((7,), [None, [0]]),
    ((3, 5), [None, [0], [1], [0, 1], []]),
    ((4, 6, 8), [None, [0], [1], [2], [0, 2], [1, 2], [0, 1]]),
    ((2, 3, 4, 5), [[1, 3], [0, 1, 3], [2], [0, 2, 3]]),
    ((33, 65), [[0], [1]]),
    ((1, 1000), [[1], None]),
    ((1000, 3), [[0], [1]]),
    ((5, 1, 7), [[1], [0, 2]]),
]


def _cases():
    for shape, axes_list in SHAPES_AXES:
        for axes in axes_list:
            for kd in (False, True):
                yield shape, axes, kd


@pytest.mark.parametrize("shape,axes,kd", list(_cases()))
@pytest.mark.parametrize("dt", ["int32", "uint8", "int64"])
def test_integer_reductions_bit_exact(shape, axes, kd, dt):
    g = rng(10)
    x = g.integers(-20 if dt != "uint8" else 0, 20, shape).astype(dt)
    for op in ["sum", "prod", "amax", "amin", "norm_l0", "norm_l1", "norm_sq"]:
        if op == "prod" and np.prod(shape) > 40:
            continue
        got = ops.reduce(op, dev(x), axes, keep_dims=kd).to_numpy()
        ref = O.reduce(op, H(x), axes, keep_dims=kd)
        np.testing.assert_array_equal(got, ref, err_msg=f"{op} {shape} {axes} kd={kd}")
    # sum<int64_t>
    got = ops.reduce("sum", dev(x), axes, keep_dims=kd, acc_dtype="int64").to_numpy()
    np.testing.assert_array_equal(got, O.reduce("sum", H(x), axes, keep_dims=kd, acc_dtype="int64"))
    # mean of integers: integer sum then double division -> bit-exact too
    got = ops.reduce("mean", dev(x), axes, keep_dims=kd).to_numpy()
    np.testing.assert_array_equal(got, O.reduce("mean", H(x), axes, keep_dims=kd))


@pytest.mark.parametrize("shape,axes,kd", list(_cases()))
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_float_reductions(shape, axes, kd, dt):
    g = rng(11)
    x = g.standard_normal(shape).astype(dt)
    xd = x.astype(np.float64)
    ax = None if axes is None else tuple(axes)
    absx = np.abs(xd).sum(axis=ax, keepdims=kd) if axes != [] else np.abs(xd)
    exact = xd.sum(axis=ax, keepdims=kd) if axes != [] else xd
    rel = 1e-6 if dt == "float32" else 1e-13
    got = ops.reduce("sum", dev(x), axes, keep_dims=kd).to_numpy()
    ref = O.reduce("sum", H(x), axes, keep_dims=kd)
    assert_close_rel(got, exact, rel, absx, "sum vs fp64")
    env = np.abs(ref.astype(np.float64) - exact) + rel * absx
    assert (np.abs(got - ref) <= env + 1e-300).all(), "sum outside the reference envelope"
    for op in ["amax", "amin"]:
        g_ = ops.reduce(op, dev(x), axes, keep_dims=kd).to_numpy()
        r_ = O.reduce(op, H(x), axes, keep_dims=kd)
        np.testing.assert_array_equal(g_, r_, err_msg=op)
    n = int(np.prod([shape[a] for a in (range(len(shape)) if axes is None else axes)])) if axes != [] else 1
    got = ops.reduce("mean", dev(x), axes, keep_dims=kd).to_numpy()
    assert_close_rel(got, exact / n, rel, absx / n, "mean")
    if n > 1:
        for ddof in (0, 1):
            vg = ops.reduce("variance", dev(x), axes, keep_dims=kd, ddof=ddof).to_numpy()
            vr = O.reduce("variance", H(x), axes, keep_dims=kd, ddof=ddof)
            assert_close_rel(vg, vr, 1e-6 if dt == "float32" else 1e-12, None, f"variance ddof={ddof}")
        sg = ops.reduce("stddev", dev(x), axes, keep_dims=kd).to_numpy()
        sr = O.reduce("stddev", H(x), axes, keep_dims=kd)
        assert_close_rel(sg, sr, 1e-6 if dt == "float32" else 1e-12, None, "stddev")
    ng = ops.reduce("norm_l2", dev(x), axes, keep_dims=kd).to_numpy()
    nr = O.reduce("norm_l2", H(x), axes, keep_dims=kd)
    assert_close_rel(ng, nr, 1e-6 if dt == "float32" else 1e-13, None, "norm_l2")


def test_reduction_of_expression_and_initial():
    g = rng(12)
    A = g.uniform(-1, 1, (40, 300)).astype(np.float32)
    b = g.standard_normal(300).astype(np.float32)
    e_d = dev(A) * dev(b) + xg.exp(-dev(A) * dev(A))
    got = ops.reduce("sum", e_d, [1]).to_numpy()
    E = O.assign(H(A) * H(b) + xg.exp(-H(A) * H(A)))
    exact = E.astype(np.float64).sum(1)
    assert_close_rel(got, exact, 1e-6, np.abs(E.astype(np.float64)).sum(1), "fused sum(E,{1})")
    x = np.arange(5 * 5 * 5 * 5, dtype=np.float64).reshape(5, 5, 5, 5)
    r = ops.reduce("sum", dev(x), [0, 2], keep_dims=True, initial=5.0).to_numpy()
    np.testing.assert_array_equal(r, x.sum(axis=(0, 2), keepdims=True) + 5)
    r = ops.reduce("prod", dev(x), [1, 2], keep_dims=True, initial=0.0).to_numpy()
    assert (r == 0).all()


def test_reduction_errors_and_edge_cases():
    a = dev(np.array([[1, 2, 3], [4, 5, 6]], np.int32))
    for axes in ([1, 0], [0, 0], [0, 2]):
        with pytest.raises(xg.XtgError) as ei:
            ops.reduce("sum", a, axes)
        assert ei.value.status == 3
    assert ops.reduce("sum", a, [-1]).to_numpy().tolist() == [6, 15]
    # zero shape
    z = dev(np.zeros((0, 1), np.int32))
    r0 = ops.reduce("sum", z, [0], keep_dims=True).to_numpy()
    assert r0.shape == (1, 1) and r0[0, 0] == 0
    r1 = ops.reduce("sum", z, [1], keep_dims=True).to_numpy()
    assert r1.shape == (0, 1)
    # empty array -> NaN mean
    e = dev(np.ones((1, 2, 0, 1), np.float64))
    assert np.isnan(ops.reduce("mean", e).to_numpy())
    r2 = ops.reduce("mean", e, [2]).to_numpy()
    assert r2.shape == (1, 2, 1) and np.isnan(r2).all()
    # uint8 sum does not overflow (result type int)
    c = dev(np.ones(1000, np.uint8))
    assert int(ops.reduce("sum", c).to_numpy()) == 1000


@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_signed_zero_and_inf_selection(dt):
    x = np.array([[0.0, -0.0, -0.0], [-0.0, 0.0, -np.inf]], dt)
    for axes in ([1], [0], None):
        for op in ("amax", "amin"):
            got = ops.reduce(op, dev(x), axes).to_numpy()
            ref = O.reduce(op, H(x), axes)
            np.testing.assert_array_equal(np.signbit(got), np.signbit(ref))
            np.testing.assert_array_equal(got, ref)
    y = np.full((4,), -np.inf, dt)
    assert ops.reduce("amax", dev(y)).to_numpy() == O.reduce("amax", H(y))


def test_float64_selection_prefilter_edges():
    """float64 amax/amin/argmax/argmin skip most FP64 compares with a 32-bit
    key of the high word: values equal in the high word, signed zeros,
    infinities, subnormals and the largest finite values must still select
    exactly like the plain fold."""
    g = rng(21)
    base = np.float64(1.5)
    hi_ties = base + np.arange(64) * np.finfo(np.float64).eps  # same high word, different low words
    specials = np.array([0.0, -0.0, np.inf, -np.inf, 5e-324, -5e-324, np.finfo(np.float64).max,
                         -np.finfo(np.float64).max, 2.2250738585072014e-308], np.float64)
    rows = []
    for r in range(40):
        v = g.permutation(np.concatenate([hi_ties, -hi_ties, specials, g.standard_normal(60)]))
        if r % 4 == 1:
            v = np.where(np.isinf(v), 0.0, v)
        if r % 4 == 2:
            v = v[g.permutation(v.size)] * 1e-310
        rows.append(v)
    x = np.stack(rows)
    for axes in ([1], [0], None):
        for op in ("amax", "amin"):
            got = ops.reduce(op, dev(x), axes).to_numpy()
            ref = O.reduce(op, H(x), axes)
            np.testing.assert_array_equal(np.signbit(got), np.signbit(ref))
            np.testing.assert_array_equal(got, ref)
    for axis in (None, 0, 1):
        for op in ("argmax", "argmin"):
            np.testing.assert_array_equal(ops.argreduce(op, dev(x), axis).to_numpy(), O.argreduce(op, H(x), axis))
    # long rows of near-equal values: the winner sits in the low word only
    y = np.broadcast_to(hi_ties, (3, 2048, 64)).reshape(3, -1).copy()
    for i in range(3):
        y[i] = y[i][g.permutation(y.shape[1])]
    for op in ("amax", "amin"):
        np.testing.assert_array_equal(ops.reduce(op, dev(y), [1]).to_numpy(), O.reduce(op, H(y), [1]))
    for op in ("argmax", "argmin"):
        np.testing.assert_array_equal(ops.argreduce(op, dev(y), 1).to_numpy(), O.argreduce(op, H(y), 1))


@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_long_row_selection_specials(dt):
    """amax / amin over long rows (split work items, block-wide groups): the
    position-free first pass hands over to the exact pass with positions
    whenever a group meets a zero at the extreme, a NaN or (float64) another
    special value — the signed zero that wins is the one the fold visits
    last, a trailing NaN wins."""
    g = rng(22)
    n = 1 << 20
    x = -np.abs(g.standard_normal((6, n))).astype(dt) - 1
    x[0, 1000] = 0.0
    x[0, n - 5000] = -0.0  # the later zero: -0
    x[1, 7] = -0.0
    x[1, n - 1] = 0.0  # +0 last
    x[2, n // 2] = np.nan
    x[2, n - 1] = np.nan  # a trailing NaN: the fold ends on it
    x[3] = g.standard_normal(n).astype(dt)  # no specials: the fast pass alone
    x[4, 123] = -np.inf
    x[5, 99] = np.inf
    for op in ("amax", "amin"):
        y = -x if op == "amin" else x
        got = ops.reduce(op, dev(y), [1]).to_numpy()
        ref = O.reduce(op, H(y), [1])
        # (a NaN result is a NaN; float64 selection returns it as a canonical NaN)
        num = ~np.isnan(ref)
        np.testing.assert_array_equal(np.signbit(got[num]), np.signbit(ref[num]), err_msg=op)
        np.testing.assert_array_equal(got, ref, err_msg=op)


# ------------------------------------------------------------------------------- arg
@pytest.mark.parametrize("dt", ["float32", "float64", "int32"])
def test_argmax_argmin(dt):
    g = rng(13)
    x = g.integers(-3, 4, (6, 37, 29)).astype(dt)  # many ties
    for op in ("argmax", "argmin"):
        for axis in (None, 0, 1, 2, -1):
            got = ops.argreduce(op, dev(x), axis).to_numpy()
            ref = O.argreduce(op, H(x), axis)
            np.testing.assert_array_equal(got, ref, err_msg=f"{op} axis={axis}")
    got = ops.argreduce("argmax", dev(x), 1, out_dtype="int32").to_numpy()
    np.testing.assert_array_equal(got, O.argreduce("argmax", H(x), 1).astype(np.int32))


@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_argmax_nan_rules(dt):
    x = np.array([[np.nan, 1, 2], [1, np.nan, 3], [2, 2, np.nan]], dt)
    for axis in (0, 1, None):
        for op in ("argmax", "argmin"):
            np.testing.assert_array_equal(ops.argreduce(op, dev(x), axis).to_numpy(), O.argreduce(op, H(x), axis))


@pytest.mark.parametrize("dt", ["float32", "int32", "float64"])
def test_argmax_column_walk_split_starts(dt):
    """Column arg-reductions split the reduced axis (here 64 splits of 64
    rows): a thread's first rows may hold NaN (skipped unless at position 0),
    -inf or ties; the compare-only update starts once every column holds a
    value.  Bit-exact against the plain fold."""
    g = rng(23)
    x = g.integers(-3, 4, (4, 4096, 64)).astype(dt)
    if dt != "int32":
        x[:, 64, :8] = np.nan        # first row of split 1
        x[:, 64:70, 8:12] = np.nan   # several leading rows
        x[:, 0, 12:14] = np.nan      # position 0: the NaN is the result
        x[:, 128, 14:16] = -np.inf
        x[:, 192:256, 16:18] = np.nan  # a whole split of NaN
    x[:, 4000, 20] = 9  # a late unique maximum
    for op in ("argmax", "argmin"):
        got = ops.argreduce(op, dev(x), 1).to_numpy()
        np.testing.assert_array_equal(got, O.argreduce(op, H(x), 1), err_msg=op)


def test_reference_argmax_kats():
    a = np.array([[5, 3, 1], [4, 4, 4]], np.float64)
    assert ops.argreduce("argmax", dev(a)).to_numpy() == 0
    np.testing.assert_array_equal(ops.argreduce("argmax", dev(a), 0).to_numpy(), [0, 1, 1])
    np.testing.assert_array_equal(ops.argreduce("argmax", dev(a), 1).to_numpy(), [0, 0])
    np.testing.assert_array_equal(ops.argreduce("argmin", dev(a), 0).to_numpy(), [1, 0, 0])
    np.testing.assert_array_equal(ops.argreduce("argmin", dev(a), 1).to_numpy(), [2, 0])
    c = np.array([[[1, 2, 3, 4]], [[4, 3, 2, 1]]], np.int32)
    np.testing.assert_array_equal(ops.argreduce("argmax", dev(c), 2).to_numpy(), [[3], [0]])
    np.testing.assert_array_equal(ops.argreduce("argmax", dev(c), 0).to_numpy(), [[1, 1, 0, 0]])


# ------------------------------------------------------------------------------- fused rows
@pytest.mark.parametrize("dt,rel", [("float32", 1e-6), ("float64", 1e-12)])
@pytest.mark.parametrize("shape", [(8, 16, 1024), (5, 3, 100), (4, 2048), (3, 5000)])
def test_row_normalize(dt, rel, shape):
    g = rng(14)
    x = g.standard_normal(shape).astype(dt)
    d = dev(x)
    out = DeviceArray.empty(shape, dt)
    xg.assign(out, (d - xg.rmean(d)) / xg.sqrt(xg.rvar(d) + 1e-5))
    xd = x.astype(np.float64)
    m = xd.mean(-1, keepdims=True)
    s = np.sqrt(xd.var(-1, keepdims=True) + 1e-5)
    exact = (xd - m) / s
    got = out.to_numpy().astype(np.float64)
    scale = (np.abs(xd) + np.abs(m)) / s
    assert_close_rel(got, exact, 4 * rel if dt == "float32" else rel, scale, "normalize")
    # the oracle follows the reference (float32 sequential row sums), so it
    # carries its own error: the GPU must sit inside that envelope
    hx = H(x)
    ref = O.assign((hx - xg.rmean(hx)) / xg.sqrt(xg.rvar(hx) + 1e-5), dtype=dt).astype(np.float64)
    env = np.abs(ref - exact) + (4 * rel if dt == "float32" else rel) * scale
    assert (np.abs(got - ref) <= env).all(), "normalize outside the reference envelope"


def _exact_row_moments(row):
    from fractions import Fraction
    v = [Fraction(float(t)) for t in row]
    s = sum(v)
    m = s / len(v)
    return s, m, sum((t - m) ** 2 for t in v)


@pytest.mark.parametrize("n", [1024, 100, 7, 3000])
def test_row_moments_float64(n):
    """float64 row sums, means and variances inside fused row trees are exact
    up to the final rounding for rows whose elements share the top binade,
    whatever the mean (no cancellation): offsets of 1e6 and 1e12 over unit
    spread, wide dynamic ranges, integer values near 2^52, subnormals; rows
    with an infinity or NaN follow IEEE arithmetic."""
    g = rng(22)
    kinds = [g.standard_normal(n), g.standard_normal(n) + 1e6, g.standard_normal(n) * 1e-3 + 1e12,
             g.standard_normal(n) * np.exp(g.uniform(-30, 30, n)),
             g.integers(-2**52, 2**52, n).astype(np.float64), g.standard_normal(n) * 1e-310,
             np.full(n, 3.25), np.zeros(n)]
    x = np.stack(kinds)
    d = dev(x)
    outs = {}
    for name, fn in [("sum", xg.rsum), ("mean", xg.rmean), ("var", xg.rvar), ("std", xg.rstd)]:
        o = DeviceArray.empty(x.shape, "float64")
        xg.assign(o, fn(d) + 0.0 * d)
        outs[name] = o.to_numpy()[:, 0]
        assert (o.to_numpy() == outs[name][:, None]).all()
    for i, row in enumerate(x):
        s, m, q = _exact_row_moments(row)
        # each element is rounded to the ulp of the row's top binade, then
        # the sum is exact and rounded once (the mean twice more)
        mx = float(np.max(np.abs(row)))
        ulp_top = np.ldexp(1.0, max(int(np.frexp(mx)[1]) - 53, -1074)) if mx > 0 else 0.0
        tol_s = n * ulp_top / 2 + 2.3e-16 * abs(float(s))
        assert abs(outs["sum"][i] - float(s)) <= tol_s, (i, outs["sum"][i], float(s))
        assert abs(outs["mean"][i] - float(m)) <= tol_s / n + 4.5e-16 * abs(float(m)), (i, outs["mean"][i], float(m))
        var = float(q / n)
        if var > 1e-290:
            assert abs(outs["var"][i] - var) <= 1e-14 * var, (i, outs["var"][i], var)
            assert abs(outs["std"][i] - np.sqrt(var)) <= 1e-14 * np.sqrt(var)
        else:
            assert abs(outs["var"][i]) <= 1e-290
    # rows with non-finite values: the IEEE path (same results as numpy)
    y = g.standard_normal((4, n))
    y[0, n // 2] = np.inf
    y[1, 0] = np.nan
    y[2, -1] = -np.inf
    y[3, n // 3] = np.inf
    y[3, n // 4] = -np.inf
    o = DeviceArray.empty(y.shape, "float64")
    xg.assign(o, xg.rmean(dev(y)) + 0.0 * dev(y))
    got = o.to_numpy()[:, 0]
    with np.errstate(invalid="ignore"):  # inf - inf in the last row: NaN expected
        want = y.mean(-1)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    np.testing.assert_array_equal(got[~np.isnan(got)], want[~np.isnan(got)])


@pytest.mark.parametrize("n", [1024, 1000])
def test_row_moments_float64_overflowing_variance(n):
    """Finite float64 rows whose squared deviations overflow (|x| ~ 1e200):
    the fixed-point moments round the variance to infinity, and the scaling
    by 1/n (by the exponent field when n is a power of two, else a multiply)
    keeps it infinite, as numpy's and the reference's float64 arithmetic do;
    the normalised row is then all zeros.  Rows near the bottom of the range
    (|x| ~ 1e-200) give a variance that underflows to 0."""
    g = rng(24)
    x = np.stack([g.standard_normal(n) * 1e200, g.standard_normal(n) * 1e-200])
    d = dev(x)
    with np.errstate(over="ignore", under="ignore"):
        want_var = x.var(-1)
        want_mean = x.mean(-1)
    assert np.isinf(want_var[0]) and want_var[1] == 0.0
    o = DeviceArray.empty(x.shape, "float64")
    xg.assign(o, xg.rvar(d) + 0.0 * d)
    got_var = o.to_numpy()[:, 0]
    assert np.isposinf(got_var[0]) and got_var[1] == 0.0, got_var
    xg.assign(o, xg.rmean(d) + 0.0 * d)
    np.testing.assert_allclose(o.to_numpy()[:, 0], want_mean, rtol=1e-14, atol=0)
    xg.assign(o, (d - xg.rmean(d)) / xg.sqrt(xg.rvar(d) + 1e-5))
    y = o.to_numpy()
    np.testing.assert_array_equal(y[0], np.zeros(n))
    exact = (x[1] - want_mean[1]) / np.sqrt(1e-5)
    np.testing.assert_allclose(y[1], exact, rtol=1e-12, atol=1e-300)


def test_row_stats_other_modes():
    g = rng(15)
    x = g.standard_normal((6, 7, 33)).astype(np.float32)
    d = dev(x)
    for fn, ref in [(lambda v: v - xg.ramax(v), lambda v: v - v.max(-1, keepdims=True)),
                    (lambda v: v / xg.rsum(v, 2), lambda v: v / v.astype(np.float64).sum((-2, -1), keepdims=True)),
                    (lambda v: xg.rstd(v, 1, 1) * 1, lambda v: np.broadcast_to(v.astype(np.float64).std(-1, ddof=1, keepdims=True), v.shape))]:
        out = DeviceArray.empty(x.shape, "float32")
        xg.assign(out, fn(d))
        r = ref(x)
        assert_close_rel(out.to_numpy(), r, 1e-5, np.abs(r) + 1e-3, "row stat")
