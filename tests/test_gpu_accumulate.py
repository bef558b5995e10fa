"""GPU accumulators (xt::cumsum / cumprod / nancumsum / nancumprod) against
the oracle and the reference's known answers.

Tolerances (stated here, checked below):
  * integer results: bit-exact (wrap-around arithmetic is associative);
  * float results folded in the sequential order — along a non-innermost
    axis, and along the innermost axis of many rows — bit-exact;
  * float results of the tile scan (a few long rows, the flattened form):
    float32 |gpu - exact| <= 2^-23 |exact| + 2^-36 * prefix sum|x| (sums;
    products 4 ulp of the exact product), float64 within the reference's own
    sequential error envelope plus 1e-15 of the prefix magnitude (rows of
    3M elements: 1e-12 of the prefix magnitude for sums, 1e-9 relative for
    products, where both folds' rounding grows with the length);
  * reproducible: the same call twice gives identical bits; the streamed
    float64 scan gives the same bits with and without pass A's lane folds.
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import XtgError, last_kernels
from xtensor_gb300.device import DeviceArray, HostArray as H
from oracle import oracle as O

from acc_kats import KATS, nan_equivalence_cases
from util import rng

pytestmark = pytest.mark.gpu


def dev(a, dtype=None):
    return DeviceArray.from_numpy(a, dtype)


@pytest.fixture
def strategy():
    def set_(v):
        xg.set_option("scan.strategy", v)
    yield set_
    xg.set_option("scan.strategy", -1)


@pytest.mark.parametrize("name", [k[0] for k in KATS])
def test_reference_kats(name):
    _, x, op, axis, expected, edt = next(k for k in KATS if k[0] == name)
    got = ops.accumulate(op, dev(x), axis).to_numpy()
    assert got.dtype == np.dtype(edt)
    assert got.shape == expected.shape
    np.testing.assert_array_equal(got, expected.astype(edt))


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int16", "int64", "uint8"])
@pytest.mark.parametrize("axis", [0, 1, 2, -1])
def test_sequential_paths_bit_exact(dt, axis):
    """Along an axis with many rows: every output folded in the reference's
    order, so floats are bit-identical to the oracle."""
    g = rng(30)
    shape = (37, 65, 129)
    if dt.startswith("float"):
        x = g.standard_normal(shape).astype(dt)
    else:
        x = g.integers(0 if dt == "uint8" else -5, 6, shape).astype(dt)
    for op in ("cumsum", "cumprod"):
        got = ops.accumulate(op, dev(x), axis).to_numpy()
        ref = O.accumulate(op, H(x), axis)
        assert got.dtype == ref.dtype
        ks = last_kernels()
        assert ks and ks[-1].split("<")[0] in ("k_scan_col", "k_scan_rows"), ks
        np.testing.assert_array_equal(got, ref, err_msg=f"{op} axis={axis}")


def _tile_tol_check(got, x, op, what):
    x64 = x.astype(np.float64)
    if op == "cumsum":
        exact = np.cumsum(x64, -1)
        pref_abs = np.cumsum(np.abs(x64), -1)
        tol = 2.0**-23 * np.abs(exact) + 2.0**-36 * pref_abs
    else:
        exact = np.cumprod(x64, -1)
        tol = 4 * 2.0**-23 * np.abs(exact) + 1e-300
    err = np.abs(got.astype(np.float64) - exact)
    assert (err <= tol).all(), f"{what}: max err {err.max()} (worst idx {np.argmax(err - tol)})"


@pytest.mark.parametrize("shape", [(3, 5000), (1, 100003), (2, 4096), (5, 1)])
def test_tile_scan_float32(shape, strategy):
    g = rng(31)
    x = g.standard_normal(shape).astype(np.float32)
    strategy(2)
    got = ops.accumulate("cumsum", dev(x), -1).to_numpy()
    assert last_kernels()[-1].startswith("k_scan_seg_apply")
    _tile_tol_check(got, x, "cumsum", "cumsum")
    # the reference's sequential float32 fold carries its own error; the tile
    # scan must sit inside that envelope
    ref = O.accumulate("cumsum", H(x), -1)
    exact = np.cumsum(x.astype(np.float64), -1)
    env = np.abs(ref - exact) + 2.0**-23 * np.abs(exact) + 2.0**-36 * np.cumsum(np.abs(x.astype(np.float64)), -1)
    assert (np.abs(got - ref) <= env).all()
    # products of values near 1 (stay finite over long rows)
    y = (1.0 + 1e-4 * g.standard_normal(shape)).astype(np.float32)
    got = ops.accumulate("cumprod", dev(y), -1).to_numpy()
    _tile_tol_check(got, y, "cumprod", "cumprod")


def test_tile_scan_int_and_float64_exact_paths(strategy):
    g = rng(32)
    strategy(2)
    xi = g.integers(-1000, 1000, (3, 20000)).astype(np.int32)
    np.testing.assert_array_equal(ops.accumulate("cumsum", dev(xi), 1).to_numpy(), O.accumulate("cumsum", H(xi), 1))
    xl = g.integers(-3, 4, (2, 9000)).astype(np.int64)
    np.testing.assert_array_equal(ops.accumulate("cumprod", dev(xl), 1).to_numpy(), O.accumulate("cumprod", H(xl), 1))
    xd = g.standard_normal((2, 30000))
    got = ops.accumulate("cumsum", dev(xd), 1).to_numpy()
    ref = O.accumulate("cumsum", H(xd), 1)
    # float64 tiles fold in FP64 in a different association than the
    # sequential reference: both are within a few ulp of the prefix magnitude
    assert (np.abs(got - ref) <= 2e-15 * np.cumsum(np.abs(xd), 1)).all()


def test_flattened_forms_and_views():
    g = rng(33)
    x = g.standard_normal((6, 7, 8)).astype(np.float64)
    d = dev(x)
    # flattened contiguous: 1-D tile scan
    got = ops.accumulate("cumsum", d, None).to_numpy()
    np.testing.assert_allclose(got, np.cumsum(x.reshape(-1)), rtol=1e-13, atol=1e-13)
    # flattened over a transposed view: evaluated into a temporary first
    t = d.transpose((2, 0, 1))
    got = ops.accumulate("cumsum", t, None).to_numpy()
    np.testing.assert_allclose(got, np.cumsum(np.ascontiguousarray(x.transpose(2, 0, 1)).reshape(-1)),
                               rtol=1e-13, atol=1e-13)
    # along an axis of a transposed view: strided leaves, sequential fold
    for ax in (0, 1, 2):
        np.testing.assert_array_equal(ops.accumulate("cumsum", t, ax).to_numpy(),
                                      O.accumulate("cumsum", H(np.ascontiguousarray(x.transpose(2, 0, 1))), ax))


def test_expression_operand_fused():
    """cumsum(A * b + C, 1) with b broadcast: the tree is evaluated inside the
    scan (no temporary), converted to the accumulation type first."""
    g = rng(34)
    A = g.standard_normal((300, 257)).astype(np.float32)
    b = g.standard_normal((257,)).astype(np.float32)
    C_ = g.standard_normal((300, 257)).astype(np.float32)
    e_dev = dev(A) * dev(b) + dev(C_)
    e_host = H(A) * H(b) + H(C_)
    for ax in (0, 1):
        np.testing.assert_array_equal(ops.accumulate("cumsum", e_dev, ax).to_numpy(),
                                      O.accumulate("cumsum", e_host, ax))
    # accumulation type argument: xt::cumsum<double>(float expression)
    got = ops.accumulate("cumsum", e_dev, 1, acc_dtype="float64").to_numpy()
    assert got.dtype == np.float64
    np.testing.assert_array_equal(got, O.accumulate("cumsum", e_host, 1, acc_dtype="float64"))


@pytest.mark.parametrize("strat", [0, 1, 2])
def test_nan_variants(strat, strategy):
    a = nan_equivalence_cases()
    strategy(strat)
    for axis in (None, 0, 1, 2):
        for op, fill, plain in (("nancumsum", 0.0, "cumsum"), ("nancumprod", 1.0, "cumprod")):
            got = ops.accumulate(op, dev(a), axis).to_numpy()
            want = O.accumulate(plain, H(np.where(np.isnan(a), fill, a)), axis)
            if axis is None or (axis == 2 and strat == 2):
                np.testing.assert_allclose(got, want, rtol=1e-14, atol=1e-14)
            else:
                np.testing.assert_array_equal(got, want)
    # inf - inf inside nancumsum stays NaN (NaN partials are not skipped)
    v = np.array([1.0, np.inf, -np.inf, 2.0, np.nan, 3.0])
    for s in (1, 2):
        strategy(s)
        np.testing.assert_array_equal(np.isnan(ops.accumulate("nancumsum", dev(v), 0).to_numpy()),
                                      np.isnan(O.accumulate("nancumsum", H(v), 0)))


def test_signed_zero_and_edges(strategy):
    z = np.array([-0.0, -0.0, -0.0], np.float64)
    for s in (1, 2):
        strategy(s)
        got = ops.accumulate("cumsum", dev(z), 0).to_numpy()
        assert np.signbit(got).all()
    strategy(0)
    one = np.array([[7.5]])
    np.testing.assert_array_equal(ops.accumulate("cumsum", dev(one), 1).to_numpy(), one)
    np.testing.assert_array_equal(ops.accumulate("cumsum", dev(one), None).to_numpy(), [7.5])
    e = DeviceArray.from_numpy(np.ones((3, 4, 0)))
    assert ops.accumulate("cumsum", e, 2).to_numpy().shape == (3, 4, 0)
    assert ops.accumulate("cumsum", e, None).to_numpy().shape == (0,)
    for ax in (3, -4):
        with pytest.raises(XtgError) as ei:
            ops.accumulate("cumsum", dev(np.ones((2, 3, 4))), ax)
        assert ei.value.status == 3
    with pytest.raises(XtgError):
        ops.accumulate("cumsum", dev(np.ones((2, 3), np.float32)), 1, out=DeviceArray.empty((2, 3), "float64"))


def test_large_tile_scan_reproducible_and_accurate():
    """2^24 float32 elements, flattened: identical bits on repeat, and within
    the stated double-float bound of the exact prefix."""
    g = rng(35)
    n = 1 << 24
    x = (g.lognormal(0, 1, n) * np.where(g.random(n) < 0.5, -1, 1)).astype(np.float32)
    d = dev(x)
    a = ops.accumulate("cumsum", d, None).to_numpy()
    b = ops.accumulate("cumsum", d, None).to_numpy()
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    exact = np.cumsum(x.astype(np.float64))
    tol = 2.0**-23 * np.abs(exact) + 2.0**-36 * np.cumsum(np.abs(x.astype(np.float64)))
    assert (np.abs(a - exact) <= tol).all()


def test_tile_scan_long_products():
    """float32 cumprod over 4.2M elements (one row cut into segments): the
    double-float states are renormalised before two of them multiply — the
    per-element chain lets lo drift to ~1e-3 of hi, and a product of two
    such states that drops lo * lo was 4.8e-4 off at the end of this row.
    Within 4 ulp of the exact prefix product; nancumprod skips NaNs."""
    g = rng(37)
    n = (1 << 22) + 12345
    y = (1.0 + 1e-5 * g.standard_normal(n)).astype(np.float32)
    got = ops.accumulate("cumprod", dev(y), None).to_numpy()
    assert last_kernels()[-1].startswith("k_scan_seg_apply")
    _tile_tol_check(got[None, :], y[None, :], "cumprod", "long cumprod")
    y[[5, n // 3]] = np.nan
    got = ops.accumulate("nancumprod", dev(y), None).to_numpy()
    _tile_tol_check(got[None, :], np.where(np.isnan(y), np.float32(1), y)[None, :], "cumprod", "long nancumprod")
    # the same row as (1, n) along axis 1 with the segmented strategy
    g2 = rng(38)
    z = (1.0 + 1e-5 * g2.standard_normal((1, n))).astype(np.float32)
    got = ops.accumulate("cumprod", dev(z), 1).to_numpy()
    _tile_tol_check(got, z, "cumprod", "long cumprod axis 1")


def test_tile_scan_strided_and_broadcast_operands(strategy):
    """The segmented scan over a strided view (every other column: the
    shared-memory path) and over a broadcast expression (the vector path)."""
    g = rng(36)
    strategy(2)
    x = g.integers(-50, 50, (3, 20001)).astype(np.int64)
    d = dev(x)
    v = d[:, ::2]
    np.testing.assert_array_equal(ops.accumulate("cumsum", v, 1).to_numpy(), np.cumsum(x[:, ::2], 1))
    b = g.integers(-5, 5, (20001,)).astype(np.int64)
    e = d * dev(b) + 3
    np.testing.assert_array_equal(ops.accumulate("cumsum", e, 1).to_numpy(), np.cumsum(x * b + 3, 1))
    f = g.standard_normal((2, 50000)).astype(np.float32)
    got = ops.accumulate("cumsum", dev(f)[:, ::3], 1).to_numpy()
    _tile_tol_check(got, np.ascontiguousarray(f[:, ::3]), "cumsum", "strided float32")


@pytest.fixture
def scan_opts():
    names = []

    def set_(name, v):
        names.append(name)
        xg.set_option(name, v)
    yield set_
    for n in names:
        xg.set_option(n, -1)


@pytest.mark.parametrize("op", ["cumsum", "cumprod", "nancumsum"])
def test_float64_streamed_scan_lane_totals(op, scan_opts, strategy):
    """float64 operands of the segmented scan stream through the apply pass's
    cp.async ring, and pass A keeps the lanes' tile folds for it (two chains
    of 8 per lane): they are the same values pass C would fold, so results are identical
    bit for bit with and without them; and close to the reference's
    sequential fold (1e-12 of the prefix magnitude for sums, 1e-9 relative
    for products of 3M factors: both folds carry rounding errors growing with
    the length; a wrong segment prefix would be off by O(1)).  Lengths that
    end inside a warp tile, several segments per row, a few long rows."""
    g = rng(61)
    # rows of an even length: 16-byte aligned rows (the streamed form);
    # 700002 = 1367 x 512 + 98 ends inside a warp tile and a lane's elements
    for shape, axis in (((3_000_001,), None), ((3, 700_002), 1)):
        if op == "cumprod":
            x = 1.0 + 1e-6 * g.standard_normal(shape)
        else:
            x = g.standard_normal(shape)
            if op == "nancumsum":
                x[..., ::997] = np.nan
        strategy(2 if axis is not None else -1)
        d = dev(x)
        on = ops.accumulate(op, d, axis).to_numpy()
        apply = last_kernels()[-1]
        assert apply.startswith("k_scan_seg_apply") and apply.endswith(", 16, true, 2>"), apply
        scan_opts("scan.lane_totals", 0)
        off = ops.accumulate(op, d, axis).to_numpy()
        assert last_kernels()[-1].endswith(", 16, false, 2>")
        xg.set_option("scan.lane_totals", -1)
        np.testing.assert_array_equal(on.view(np.uint64), off.view(np.uint64))
        ref = O.accumulate(op, H(x), axis)
        xs = np.where(np.isnan(x), 0.0, x) if op == "nancumsum" else x
        if op == "cumprod":
            assert (np.abs(on - ref) <= 1e-9 * np.abs(ref)).all()
        else:
            mag = np.cumsum(np.abs(xs), -1 if axis is not None else None).reshape(on.shape)
            assert (np.abs(on - ref) <= 1e-12 * mag).all()


def test_streamed_and_register_forms_agree(scan_opts):
    """The streamed apply pass (plain contiguous float32 / int32 operands,
    tiles of 32 x 16 through shared memory) and the register form (tiles of
    32 x 8) fold in different associations: integers are equal, float32
    both within the double-float bound of the exact prefix."""
    g = rng(62)
    n = (1 << 22) + 777
    xi = g.integers(-1000, 1000, n).astype(np.int32)
    x = g.standard_normal(n).astype(np.float32)
    outs = {}
    for mode in (1, 0):
        scan_opts("scan.async", mode)
        outs[mode] = (ops.accumulate("cumsum", dev(xi), None).to_numpy(),
                      ops.accumulate("cumsum", dev(x), None).to_numpy())
        assert last_kernels()[-1].endswith(", 3, 16, false, 1>" if mode else ", 0, 8, false, 1>"), last_kernels()[-1]
    np.testing.assert_array_equal(outs[1][0], outs[0][0])
    np.testing.assert_array_equal(outs[1][0], np.cumsum(xi.astype(np.int64)).astype(np.int32))
    exact = np.cumsum(x.astype(np.float64))
    tol = 2.0**-23 * np.abs(exact) + 2.0**-36 * np.cumsum(np.abs(x.astype(np.float64)))
    for mode in (1, 0):
        assert (np.abs(outs[mode][1] - exact) <= tol).all(), mode


def test_cached_plan_replay_after_smaller_call():
    """Pass B stages a row's segment totals in dynamic shared memory sized by
    the call (2^24 elements: ~4.7K segments, above 48 KiB; 10^5 elements: a
    few KiB).  A kernel's dynamic limit is only ever raised, so the large
    call's cached plan still launches after the small call configured the
    same kernel for less, and gives the same bits."""
    g = rng(63)
    big = g.standard_normal(1 << 24).astype(np.float32)
    small = g.standard_normal(100_000).astype(np.float32)
    db, ds = dev(big), dev(small)
    ob, os_ = DeviceArray.empty((big.size,), "float32"), DeviceArray.empty((small.size,), "float32")
    first = ops.accumulate("cumsum", db, None, out=ob).to_numpy()
    ops.accumulate("cumsum", ds, None, out=os_)
    again = ops.accumulate("cumsum", db, None, out=ob).to_numpy()  # replayed from the plan cache
    np.testing.assert_array_equal(first.view(np.uint32), again.view(np.uint32))
    exact = np.cumsum(small.astype(np.float64))
    tol = 2.0**-23 * np.abs(exact) + 2.0**-36 * np.cumsum(np.abs(small.astype(np.float64)))
    assert (np.abs(os_.to_numpy() - exact) <= tol).all()
