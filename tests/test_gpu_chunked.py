"""Chunked arrays over device chunks (xtg_chunked_assign / _to_dense / _reduce).

The reference's own tests (test/test_xchunked_array.cpp, test_xchunked_view.cpp)
restated on device chunks, then parity with the oracle: a chunked
assignment must store, in every chunk's valid region, exactly what the
oracle's dense assignment of the same expression gives (bit for bit for
+ - * / and conversions), leave the padding of edge chunks untouched, and
read back (to a dense array) bit for bit.  Reductions of a chunked array:
integer results equal the oracle's; float64 results within 1e-11 of the
oracle's, relative to the largest result (chunks associate the sums
differently from the plain reducer's sequential fold).
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.chunked import ChunkedArray, as_chunked_assign, chunked_reduce
from xtensor_gb300.device import DeviceArray, HostArray
from oracle import chunked as OC
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def chunks_numpy(a: ChunkedArray):
    return [c.to_numpy() for c in a.chunks]


# ---------------------------------------------------------------- reference tests
def test_indexed_access():
    # test_xchunked_array.cpp:20-44
    xg.init(0)
    a = ChunkedArray((10, 10, 10), (2, 3, 4), "float64")
    a[3, 9, 8] = 1.0
    assert a[3, 9, 8] == 1.0
    a[3, 9, 8] = 2.0
    assert a[3, 9, 8] == 2.0
    a.assign(xg.scalar(3.0) + 0 * DeviceArray.from_numpy(np.zeros((10, 10, 10))))
    assert (a.to_numpy() == 3.0).all()


def test_assign_expression():
    # test_xchunked_array.cpp:46-126
    xg.init(0)
    val = 3.0
    a1 = ChunkedArray((2, 2, 2), (2, 3, 4), "float64")
    a1.assign(xg.scalar(val) + DeviceArray.from_numpy(np.zeros((2, 2, 2))))
    assert (a1.to_numpy() == val).all()
    a2 = ChunkedArray((32, 10, 10), (2, 3, 4), "float64")
    a2.assign(xg.scalar(val) + DeviceArray.from_numpy(np.zeros((32, 10, 10))))
    assert (a2.to_numpy() == val).all()
    a2 += a2
    assert (a2.to_numpy() == 2 * val).all()
    a2 += 2.0
    assert (a2.to_numpy() == 2 * val + 2).all()
    a3 = np.arange(1.0, 10.0).reshape(3, 3)
    a4 = ChunkedArray.from_numpy(a3, (2, 2))
    np.testing.assert_array_equal(a4.to_numpy().ravel(), np.arange(1.0, 10.0))
    a5 = ChunkedArray.from_expr(a4)  # in_memory_chunked_array(a4): a4's chunk shape
    assert a5.chunk_shape == (2, 2)
    a6 = ChunkedArray.from_expr(DeviceArray.from_numpy(a3))  # chunked_array(a3): one chunk
    assert a6.chunk_shape == (3, 3)
    a7 = ChunkedArray((3, 3), (1, 2), "float64")
    a7.assign(DeviceArray.from_numpy(a3))
    assert all(c.shape == (1, 2) for c in a7.chunks)
    np.testing.assert_array_equal(a7.to_numpy(), a3)


def test_noalias_and_chunk_iterator():
    # test_xchunked_array.cpp:128-168
    xg.init(0)
    b = np.arange(1000, dtype=np.float64).reshape(10, 10, 10)
    a = ChunkedArray((10, 10, 10), (2, 2, 2), "float64")
    a.assign(DeviceArray.from_numpy(b))
    np.testing.assert_array_equal(a.to_numpy(), b)
    items = list(a.chunk_items())
    n = 0
    for i in range(5):
        for j in range(5):
            for k in range(5):
                gc, ch, sl = items[n]
                assert gc == (i, j, k)
                assert ch.to_numpy()[0, 0, 0] == a[2 * i, 2 * j, 2 * k]
                n += 1
    assert items[2][1].to_numpy()[0, 0, 0] == a[0, 0, 4]


def test_chunked_view_assign():
    # test_xchunked_view.cpp:33-63
    xg.init(0)
    a = np.arange(1.0, 13.0).reshape(3, 4)
    b = DeviceArray.empty((3, 4), "float64")
    as_chunked_assign(b, (1, 2), DeviceArray.from_numpy(a))
    np.testing.assert_array_equal(b.to_numpy(), a)
    ref = np.arange(1000, dtype=np.float64).reshape(10, 10, 10)
    ca = ChunkedArray((10, 10, 10), (2, 3, 4), "float64")
    ca.assign(DeviceArray.from_numpy(ref))  # as_chunked(a, chunk_shape) = ref
    bb = DeviceArray.empty((10, 10, 10), "float64")
    as_chunked_assign(bb, (2, 3, 4), ca)  # as_chunked(b, chunk_shape) = a
    np.testing.assert_array_equal(ca.to_numpy(), ref)
    np.testing.assert_array_equal(bb.to_numpy(), ref)


# ---------------------------------------------------------------- parity with the oracle
# chunk classes per case: 8 (edges along three dims, scalar), 8, 1 (whole
# chunks, vectors), 2 (an edge of 40 along the vectorised dim), 8, 1 (one chunk
# larger than the array), 4 (vectorised, with edges), 16 (more classes than one
# launch holds: padded chunks with extent tests)
CASES = [((37, 70, 45), (8, 16, 16)), ((37, 70, 45), (5, 9, 7)), ((64, 128), (16, 64)), ((1000,), (96,)),
         ((3, 5, 7, 9), (2, 2, 4, 3)), ((8, 8), (16, 16)), ((50, 1000), (16, 96)), ((3, 5, 7, 9, 11), (2, 2, 4, 3, 5))]


@pytest.mark.parametrize("shape,cs", CASES)
@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "bfloat16"])
def test_expression_into_chunks_matches_oracle(shape, cs, dt):
    xg.init(0)
    g = np.random.default_rng(61)
    if dt == "bfloat16":
        from util import f32_to_bf16_bits
        x = f32_to_bf16_bits(g.standard_normal(shape).astype(np.float32))
        y = f32_to_bf16_bits(g.standard_normal(shape[-1:]).astype(np.float32))
    elif dt.startswith("float"):
        x = g.standard_normal(shape).astype(dt)
        y = (g.random(shape[-1:]) + 0.5).astype(dt)
    else:
        x = g.integers(-1000, 1000, shape).astype(dt)
        y = g.integers(1, 50, shape[-1:]).astype(dt)
    dx, dy = DeviceArray.from_numpy(x, dt), DeviceArray.from_numpy(y, dt)
    hx, hy = HostArray(x, dt), HostArray(y, dt)
    f = (lambda u, v: u * v - u + 2) if dt != "int32" else (lambda u, v: u * v - u / v)
    code = O.expr_dtype(f(hx, hy))
    ref = O.assign(f(hx, hy))
    a = ChunkedArray(shape, cs, code)
    # a sentinel in every buffer: the padding of edge chunks must survive
    zero = DeviceArray.from_numpy(np.zeros(cs, np.int32))
    for c in a.chunks:
        xg.assign(c, zero + 77)
    sentinel = chunks_numpy(a)
    a.assign(f(dx, dy))
    got = chunks_numpy(a)
    want = OC.assign_chunks(sentinel, ref, cs)
    for u, v in zip(got, want):
        assert u.tobytes() == v.tobytes()
    np.testing.assert_array_equal(a.to_numpy(), ref)
    # chunked operands of the same grid: a * 2 + a, in place
    b = ChunkedArray.from_expr(f(dx, dy), cs)
    b.assign(b * 2 + a)
    np.testing.assert_array_equal(b.to_numpy(), O.assign(HostArray(ref) * 2 + HostArray(ref)))


def test_reading_into_a_strided_destination():
    xg.init(0)
    g = np.random.default_rng(62)
    x = g.standard_normal((30, 50)).astype(np.float32)
    a = ChunkedArray.from_numpy(x, (7, 16))
    big = DeviceArray.from_numpy(np.zeros((60, 50), np.float32))
    a.to_device(big[::2])
    np.testing.assert_array_equal(big.to_numpy()[::2], x)
    np.testing.assert_array_equal(big.to_numpy()[1::2], 0)


def separate_chunks(x, cs):
    """A chunked array whose chunks are separate allocations (not at equal
    distances: the reductions take the chunk-by-chunk path)."""
    from xtensor_gb300.chunked import grid_shape
    import math
    n = math.prod(grid_shape(x.shape, cs))
    chunks = [DeviceArray.empty(cs, x.dtype) for _ in range(n)]
    a = ChunkedArray(x.shape, cs, x.dtype, chunks=chunks)
    a.assign(DeviceArray.from_numpy(x))
    return a


@pytest.mark.parametrize("alloc", ["slab", "separate"])
@pytest.mark.parametrize("op", ["sum", "prod", "amax", "amin", "mean", "variance", "stddev", "norm_l1", "norm_l2",
                                "norm_linf", "norm_sq"])
@pytest.mark.parametrize("axes,kd", [(None, False), ([0], False), ([1, 2], False), ([0, 2], True), ([2], True)])
def test_reductions_match_oracle(op, axes, kd, alloc):
    xg.init(0)
    g = np.random.default_rng(63)
    shape, cs = (13, 22, 17), (4, 8, 5)
    xi = g.integers(-20, 21, shape).astype(np.int32) if op != "prod" else g.integers(1, 3, shape).astype(np.int32)
    xf = g.standard_normal(shape)
    if op == "prod":
        xf = 1 + 0.01 * xf
    for x in (xi, xf):
        a = ChunkedArray.from_numpy(x, cs) if alloc == "slab" else separate_chunks(x, cs)
        got = chunked_reduce(op, a, axes=axes, keep_dims=kd).to_numpy()
        ref = O.reduce(op, HostArray(x), axes=axes, keep_dims=kd)
        assert got.shape == ref.shape and got.dtype == ref.dtype
        if np.issubdtype(ref.dtype, np.integer):
            np.testing.assert_array_equal(got, ref)
        else:
            np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-11 * max(1.0, float(np.max(np.abs(ref)))))


def test_errors():
    xg.init(0)
    a = ChunkedArray((10, 10), (3, 4), "float32")
    b = ChunkedArray((10, 10), (5, 5), "float32")
    with pytest.raises(xg.XtgError) as ei:
        a.assign(b * 2)
    assert ei.value.status == 9  # another chunk grid
    with pytest.raises(xg.XtgError) as ei:
        a.assign(DeviceArray.from_numpy(np.ones((10, 11), np.float32)))
    assert ei.value.status == 5
    from xtensor_gb300.chunked import _sigs
    assert _sigs().xtg_chunked_reduce(None, None, None, None) == 1  # null arguments
    with pytest.raises(xg.XtgError) as ei:
        chunked_reduce("sum", a, axes=[2])
    assert ei.value.status == 3  # axis out of bounds
