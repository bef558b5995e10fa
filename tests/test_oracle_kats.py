"""The oracle pinned to the reference's own golden vectors and known-answer
tests (CPU only).  Each case cites the reference test it restates."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300.device import HostArray as H
from oracle import oracle as O

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "xmath_reducers.json").read_text())


# ---- numpy-generated golden vectors (test/test_extended_xmath_reducers.cpp) -------
def test_golden_var_std():
    """TEST(xtest_extended_xmath, var_std): np.var/np.std of a (4,5,6,7) array."""
    g = GOLDEN["var_std"]
    a = np.array(g["a"], dtype=np.float64)
    ha = H(a)
    rtol = 1e-12
    np.testing.assert_allclose(O.reduce("variance", ha), g["vr_all"], rtol=rtol)
    np.testing.assert_allclose(O.reduce("variance", ha, ddof=1), g["vr_all_ddof"], rtol=rtol)
    np.testing.assert_allclose(O.reduce("stddev", ha), g["st_all"], rtol=rtol)
    np.testing.assert_allclose(O.reduce("variance", ha, [0, 2]), np.array(g["vr"]), rtol=rtol)
    np.testing.assert_allclose(O.reduce("variance", ha, [0, 2], ddof=1), np.array(g["vr_ddof"]), rtol=rtol)
    np.testing.assert_allclose(O.reduce("stddev", ha, [0, 2]), np.array(g["st"]), rtol=rtol)


def test_golden_weighted_average_through_sums():
    """TEST(xtest_extended_xmath, average): sum(a*w, {0,1}) / sum(w, {0,1})."""
    g = GOLDEN["average"]
    a = np.array(g["a"])
    w = np.array(g["w"])
    num = O.reduce("sum", H(a) * H(w), [0, 1])
    den = O.reduce("sum", H(w), [0, 1])
    np.testing.assert_allclose(num / den, np.array(g["av"]), rtol=1e-12)


# ---- test/test_xreducer.cpp ---------------------------------------------------------------
def features():
    """xreducer_features (test_xreducer.cpp:54-82): ones(3,2,4,6,5) with 2s planted."""
    a = np.ones((3, 2, 4, 6, 5))
    for i in range(2):
        for j in range(6):
            a[1, i, 1, j, 1] = 2
    return a


def test_kat_sum_axes_and_all():
    a = features()
    res = O.reduce("sum", H(a), [1, 3])  # test_xreducer.cpp:355-362
    exp = 12 * np.ones((3, 4, 5))
    exp[1, 1, 1] = 24
    np.testing.assert_array_equal(res, exp)
    assert O.reduce("sum", H(a)) == 732  # :475-481


def test_kat_sum_tensor_sugar_and_uint8():
    m = np.array([[1, 2], [3, 4]], np.float64)
    np.testing.assert_array_equal(O.reduce("sum", H(m), [0]), [4, 6])  # :390-397
    u = np.ones((2, 4))
    np.testing.assert_array_equal(O.reduce("sum", H(u), [0]), 2 * np.ones(4))  # :442-473
    np.testing.assert_array_equal(O.reduce("sum", H(u), [-1]), 4 * np.ones(2))
    c = np.ones(1000, np.uint8)
    r = O.reduce("sum", H(c))
    assert r == 1000 and r.dtype == np.int32  # no overflow: uint8 + uint8 is int


def test_kat_prod_long_long():
    c = 2 * np.ones(34, np.uint8)  # :507-512
    assert O.reduce("prod", H(c), acc_dtype="int64") == 1 << 34


def test_kat_mean():
    x = np.array([[-1.0, 0.0], [1.0, 0.0]])  # :542-570
    assert O.reduce("mean", H(x)) == 0.0
    np.testing.assert_array_equal(O.reduce("mean", H(x), [0]), [0.0, 0.0])
    np.testing.assert_array_equal(O.reduce("mean", H(x), [1]), [-0.5, 0.5])
    assert O.reduce("mean", H(np.array([1, 2], np.uint8))) == 1.5


def test_kat_immediate_equals_lazy_axis_sets():
    """:704-771 — every axis set of arange(27).reshape(3,3,3) and (4,3,6,2,7)."""
    for shape, sets in [((3, 3, 3), [None, [1], [0, 2], [1, 2]]),
                        ((4, 3, 6, 2, 7), [None, [1], [0, 2], [1, 2], [1, 3, 4], [0, 1, 4], [0, 1, 3], [0, 2, 3], [1, 2, 3]])]:
        a = np.arange(int(np.prod(shape)), dtype=np.float64).reshape(shape)
        for ax in sets:
            got = O.reduce("sum", H(a), ax)
            np.testing.assert_array_equal(got, a.sum(axis=None if ax is None else tuple(ax)))


def test_kat_chaining_reducers():
    a = np.array([[1.0, 2.0], [3.0, 4.0]])  # :773-781
    s = O.reduce("sum", H(a), [0])
    b = O.assign(H(a) - H(s))
    np.testing.assert_array_equal(O.reduce("sum", H(b), [0]), [-4.0, -6.0])


def test_kat_keep_dims_and_initial():
    a = np.arange(5 * 5 * 5 * 5, dtype=np.float64).reshape(5, 5, 5, 5)  # :964-1018
    r = O.reduce("sum", H(a), [0, 1], keep_dims=True)
    assert r.shape == (1, 1, 5, 5)
    r5 = O.reduce("sum", H(a), [0, 2], keep_dims=True, initial=5.0)
    np.testing.assert_array_equal(r5, O.reduce("sum", H(a), [0, 2], keep_dims=True) + 5)
    assert (O.reduce("prod", H(a), [1, 2], keep_dims=True, initial=0.0) == 0).all()
    assert O.reduce("sum", H(a), keep_dims=True).shape == (1, 1, 1, 1)
    assert O.reduce("sum", H(a)).shape == ()


def test_kat_ones_first_empty_axes_zero_shape_empty_array():
    a = np.ones((1, 1, 2, 4), np.int32)  # :1020-1031
    np.testing.assert_array_equal(O.reduce("sum", H(a), [1], keep_dims=True), a)
    np.testing.assert_array_equal(O.reduce("sum", H(a), [1, 2], keep_dims=True), [[[[2, 2, 2, 2]]]])
    b = np.array([[1, 2, 3], [4, 5, 6]], np.int32)  # :1033-1042
    np.testing.assert_array_equal(O.reduce("sum", H(b), []), b)
    z = np.zeros((0, 1), np.int32)  # :1044-1062
    r0 = O.reduce("sum", H(z), [0], keep_dims=True)
    assert r0.shape == (1, 1) and r0[0, 0] == 0
    assert O.reduce("sum", H(z), [1], keep_dims=True).shape == (0, 1)
    e = np.ones((1, 2, 0, 1))  # :1064-1079
    assert np.isnan(O.reduce("mean", H(e)))
    r2 = O.reduce("mean", H(e), [2])
    assert r2.shape == (1, 2, 1) and np.isnan(r2).all()


def test_kat_axis_errors():
    a = np.ones((3, 2), np.int32)  # :213-220, :1081-1088
    O.reduce("sum", H(a), [0, 1])
    for ax in ([0, 0], [1, 0], [1, 1], [0, 2]):
        with pytest.raises(O.OracleError) as ei:
            O.reduce("sum", H(a), ax)
        assert ei.value.status == 3


# ---- test/test_xnorm.cpp:97-187 --------------------------------------------------------------
def test_kat_norms():
    a = -np.ones(9, np.int32)
    assert O.reduce("norm_l0", H(a)) == 9
    assert O.reduce("norm_l1", H(a)) == 9
    assert O.reduce("norm_sq", H(a)) == 9
    assert O.reduce("norm_l2", H(a)) == 3.0
    assert O.reduce("norm_linf", H(a)) == 1
    m = np.array([[-1.0, 2.0], [-3.0, 4.0]])
    assert O.reduce("norm_l0", H(m)) == 4
    assert O.reduce("norm_l1", H(m)) == 10.0
    assert O.reduce("norm_sq", H(m)) == 30.0
    assert O.reduce("norm_linf", H(m)) == 4.0


# ---- test/test_xsort.cpp:217-281 -------------------------------------------------------------
def test_kat_argmin_argmax():
    a = np.array([[5, 3, 1], [4, 4, 4]], np.float64)
    assert O.argreduce("argmin", H(a)) == 2
    np.testing.assert_array_equal(O.argreduce("argmin", H(a), 0), [1, 0, 0])
    np.testing.assert_array_equal(O.argreduce("argmin", H(a), 1), [2, 0])
    b = np.array([1, 3, 4, -100], np.float64)
    assert O.argreduce("argmin", H(b)) == 3 and O.argreduce("argmin", H(b), 0) == 3
    assert O.argreduce("argmax", H(a)) == 0
    np.testing.assert_array_equal(O.argreduce("argmax", H(a), 0), [0, 1, 1])
    np.testing.assert_array_equal(O.argreduce("argmax", H(a), 1), [0, 0])
    c = np.array([[[1, 2, 3, 4]], [[4, 3, 2, 1]]], np.int32)
    np.testing.assert_array_equal(O.argreduce("argmax", H(c), 2), [[3], [0]])
    np.testing.assert_array_equal(O.argreduce("argmax", H(c), 0), [[1, 1, 0, 0]])
    np.testing.assert_array_equal(O.argreduce("argmax", H(c), 1), [[0, 0, 0, 0], [0, 0, 0, 0]])
    ya = np.array([1, 0, 3, 2, 2], np.float64)
    assert O.argreduce("argmax", H(ya)) == 2 and O.argreduce("argmin", H(ya)) == 1
    assert O.argreduce("argmax", H(np.array([0.0, 1.0, 0.0]))) == 1  # xtensor#2568


# ---- test/test_xmath.cpp:379-446: exp / sqrt / square against std:: ----------------------------
def test_kat_math_functions():
    x = np.array([0.5, 1.0, 2.25, 4.0], np.float64)
    np.testing.assert_array_equal(O.assign(xg.exp(H(x))), np.exp(x))
    np.testing.assert_array_equal(O.assign(xg.sqrt(H(x))), np.sqrt(x))
    np.testing.assert_array_equal(O.assign(xg.square(H(x))), x * x)


# ---- two implementations of the C++ type rules agree ----------------------------------------------
def test_type_rules_library_vs_oracle():
    dts = ["bool", "int8", "uint8", "int16", "uint16", "int32", "uint32", "int64", "uint64", "float32", "float64"]
    arrs = {d: np.zeros((2, 3), dtype=xg.np_dtype(xg.dtype_code(d))) for d in dts}
    for da in dts:
        for db in dts:
            a, b = H(arrs[da], da), H(arrs[db], db)
            for e in (a + b, a * b, xg.maximum(a, b), xg.where(a < b, a, b), -a, xg.exp(a), xg.square(b)):
                assert xg.expr_dtype(e) == O.expr_dtype(e), (da, db)


def test_broadcast_rules_library_vs_oracle():
    g = np.random.default_rng(0)
    for _ in range(200):
        r1, r2 = g.integers(0, 4, 2)
        s1 = tuple(int(v) for v in g.choice([1, 2, 3], r1))
        s2 = tuple(int(v) for v in g.choice([1, 2, 3], r2))
        a, b = H(np.zeros(s1, np.float32)), H(np.zeros(s2, np.float32))
        try:
            want = np.broadcast_shapes(s1, s2)
        except ValueError:
            want = None
        if want is None:
            with pytest.raises(xg.XtgError) as ei:
                xg.broadcast_shape(a + b)
            assert ei.value.status == 2
        elif s1 or s2:
            assert xg.broadcast_shape(a + b) == want == O.broadcast_shape(a + b)


# ---- test/test_xaccumulator.cpp, test/test_xnan_functions.cpp:152-172 -------------------------
@pytest.mark.parametrize("name", [k[0] for k in __import__("acc_kats").KATS])
def test_kat_accumulators(name):
    from acc_kats import KATS
    _, x, op, axis, expected, edt = next(k for k in KATS if k[0] == name)
    got = O.accumulate(op, H(x), axis)
    assert got.dtype == np.dtype(edt), (got.dtype, edt)
    assert got.shape == expected.shape
    np.testing.assert_array_equal(got, expected.astype(edt))


def test_kat_nan_accumulators_and_errors():
    from acc_kats import nan_equivalence_cases
    a = nan_equivalence_cases()
    for axis in (None, 0, 1, 2):
        np.testing.assert_array_equal(O.accumulate("nancumsum", H(a), axis),
                                      O.accumulate("cumsum", H(np.where(np.isnan(a), 0.0, a)), axis))
        np.testing.assert_array_equal(O.accumulate("nancumprod", H(a), axis),
                                      O.accumulate("cumprod", H(np.where(np.isnan(a), 1.0, a)), axis))
    # xt::cumsum<double>(float) accumulates in double
    f = np.array([[0.1, 0.2], [0.3, 0.4]], np.float32)
    got = O.accumulate("cumsum", H(f), 1, acc_dtype="float64")
    assert got.dtype == np.float64
    np.testing.assert_array_equal(got, np.cumsum(f.astype(np.float64), 1))
    # an axis outside the expression: std::runtime_error
    for ax in (3, -4):
        with pytest.raises(O.OracleError) as ei:
            O.accumulate("cumsum", H(np.ones((2, 3, 4))), ax)
        assert ei.value.status == 3
