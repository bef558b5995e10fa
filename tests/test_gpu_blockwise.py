"""xt::blockwise reducers on the GPU against the blockwise restatement
(oracle/blockwise.py, itself pinned to the reference's test) and the plain
oracle reducers: input in device memory, in pageable host memory and in
pinned host memory, one slab and many slabs (the slab dimension reduced and
kept), every op, keep_dims, float inputs, a 1 GiB host input, errors.

Tolerances (stated here, checked below): integer results and integer-valued
means bit-exact; variance / stddev of the reference's int case rtol 1e-12;
float inputs: float64 rtol 1e-12, float32 rtol 2e-5 (sums over slabs and
tree sums inside a slab associate differently than the reference's block
fold; float32 powers are computed in float32 under the default fp32_compute
option), each relative to the same reduction of |x|; amin / amax / linf
exact."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import XtgError, lib
from xtensor_gb300.device import DeviceArray, HostArray as H
from oracle import blockwise as B
from oracle import oracle as O

from blockwise_cases import AXES, BLOCK, OPS, P_OPS, input_exp
from util import rng

pytestmark = pytest.mark.gpu

EXACT = {"sum", "prod", "amin", "amax", "mean", "norm_l0", "norm_l1", "norm_sq", "norm_linf"}


@pytest.fixture
def slab():
    def set_(nbytes):
        xg.set_option("blockwise.slab_bytes", nbytes)
    yield set_
    xg.set_option("blockwise.slab_bytes", 512 << 20)


class Pinned:
    """A numpy array over page-locked host memory."""

    def __init__(self, a: np.ndarray):
        self.p = C.c_void_p()
        assert lib().xtg_host_alloc(C.byref(self.p), max(a.nbytes, 1)) == 0
        buf = (C.c_char * max(a.nbytes, 1)).from_address(self.p.value)
        self.a = np.frombuffer(buf, dtype=a.dtype, count=a.size).reshape(a.shape)
        self.a[...] = a

    def close(self):
        lib().xtg_host_free(self.p)


def _check(op, got, want):
    assert got.dtype == want.dtype and got.shape == want.shape, (op, got.dtype, want.dtype, got.shape, want.shape)
    if op in EXACT:
        np.testing.assert_array_equal(got, want, err_msg=op)
    else:
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=0, err_msg=op)


@pytest.mark.parametrize("where", ["device", "pageable", "pageable_ring", "pinned"])
@pytest.mark.parametrize("keep_dims", [True, False])
def test_reference_case_all_ops(where, keep_dims, slab):
    """test_xblockwise_reducer.cpp:95-215 on the GPU: shape (21, 10, 5),
    blocks (5, 4, 2), six axis sets; slabs of one block row (1000 bytes).
    Pageable input is page-locked in place for the call, or (ring) copied
    through the pinned staging ring."""
    x = input_exp()
    slab(1000)
    xg.set_option("blockwise.register_host", 0 if where == "pageable_ring" else 1)
    pin = Pinned(x) if where == "pinned" else None
    src = DeviceArray.from_numpy(x) if where == "device" else (pin.a if pin else x)
    try:
        for axes in AXES:
            for op in OPS + P_OPS:
                got = ops.blockwise(op, src, BLOCK, list(axes), keep_dims).to_numpy()
                want = B.blockwise(op, x, BLOCK, list(axes), keep_dims)
                _check(op, got, want)
                if op in EXACT:  # and the plain reducer, as the reference's test
                    np.testing.assert_array_equal(got, O.reduce(op, H(x), list(axes), keep_dims))
    finally:
        xg.set_option("blockwise.register_host", 1)
        if pin:
            pin.close()


@pytest.mark.parametrize("dt", ["float32", "float64", "int64", "uint8", "int16"])
@pytest.mark.parametrize("order", ["C", "F"])
def test_random_inputs_many_slabs(dt, order, slab):
    g = rng(50)
    shape = (37, 29, 65)
    if dt.startswith("float"):
        x = g.standard_normal(shape).astype(dt)
    else:
        x = g.integers(0 if dt == "uint8" else -50, 50, shape).astype(dt)
    x = np.asfortranarray(x) if order == "F" else x
    block = (8, 7, 16)
    slab(4096)  # many slabs along the outermost dimension (axis 2 for F order)
    rt = 2e-5 if dt == "float32" else 1e-12
    xc = np.ascontiguousarray(x)
    ax = np.abs(xc.astype(np.float64))
    for axes in [(0,), (2,), (0, 2), (1,), (0, 1, 2)]:
        a_ = list(axes)
        # |err| <= rt * (the same reduction of |x|): float terms round alike,
        # the association of the sums differs
        scale = {"sum": B.blockwise("sum", ax, block, a_), "mean": B.blockwise("mean", ax, block, a_),
                 "variance": B.blockwise("mean", ax * ax, block, a_), "norm_l2": B.blockwise("norm_l2", ax, block, a_),
                 "norm_lp_to_p": B.blockwise("norm_lp_to_p", ax, block, a_, p=3.0),
                 "norm_lp": B.blockwise("norm_lp", ax, block, a_, p=2.0)}
        for op in ["sum", "mean", "amax", "variance", "norm_l2", "norm_linf", "norm_lp_to_p", "norm_lp"]:
            p = 3.0 if op == "norm_lp_to_p" else 2.0
            got = ops.blockwise(op, x, block, a_, False, p=p).to_numpy()
            want = B.blockwise(op, xc, block, a_, False, p=p)
            assert got.dtype == want.dtype and got.shape == want.shape
            if op in ("amax", "norm_linf") or (op in EXACT and not dt.startswith("float")):
                np.testing.assert_array_equal(got, want, err_msg=f"{op} {axes}")
            else:
                err = np.abs(got.astype(np.float64) - want.astype(np.float64))
                assert (err <= rt * scale[op] + 1e-300).all(), f"{op} {axes}: {np.max(err / (scale[op] + 1e-300))}"


def test_large_host_input_streams(slab):
    """1 GiB float32 in pageable host memory, slabs of 128 MiB: sums over the
    slab dimension (merged across slabs) and over the others (disjoint
    slabs), against float64 numpy."""
    g = rng(51)
    x = g.standard_normal((256, 1024, 1024), dtype=np.float32)
    slab(128 << 20)
    s0 = ops.blockwise("sum", x, (16, 256, 256), [0]).to_numpy()
    np.testing.assert_allclose(s0, x.sum(0, dtype=np.float64), rtol=1e-5, atol=1e-4)
    m2 = ops.blockwise("mean", x, (16, 256, 256), [1, 2]).to_numpy()
    np.testing.assert_allclose(m2, x.mean((1, 2), dtype=np.float64), rtol=1e-5, atol=1e-7)
    v = ops.blockwise("variance", x, (16, 256, 256), [0, 1, 2]).to_numpy()
    np.testing.assert_allclose(v, x.var(dtype=np.float64), rtol=1e-5)
    # pinned: the same through one DMA per slab
    pin = Pinned(x[:64])
    try:
        a = ops.blockwise("amax", pin.a, (16, 256, 256), [0, 2]).to_numpy()
        np.testing.assert_array_equal(a, x[:64].max((0, 2)))
    finally:
        pin.close()


def test_errors():
    x = input_exp()
    with pytest.raises(XtgError) as e:
        rd_op = "sum"
        a = H(x).xtg_array()
        from xtensor_gb300.ops import make_desc
        rd = make_desc(rd_op, [0], initial=3)
        out = DeviceArray.empty((10, 5), "int32")
        o = out.xtg_array()
        bs = (C.c_int64 * 8)(*BLOCK)
        xg.check(lib().xtg_blockwise_reduce(C.byref(a), bs, C.byref(rd), 2.0, C.byref(o), None))
    assert e.value.status == 9
    with pytest.raises(XtgError) as e:
        ops.blockwise("sum", x, BLOCK, [0], out=DeviceArray.empty((10, 5), "float32"))
    assert e.value.status == 1
    with pytest.raises(XtgError) as e:
        ops.blockwise("sum", x, BLOCK, [0], out=DeviceArray.empty((10, 4), "int32"))
    assert e.value.status == 5
    with pytest.raises(XtgError) as e:
        ops.blockwise("sum", x[:, ::2], BLOCK, [0])  # a host view with gaps
    assert e.value.status == 9
    with pytest.raises(XtgError, match="p must be nonzero"):
        ops.blockwise("norm_lp", x, BLOCK, [0], p=0.0)
    with pytest.raises(XtgError) as e:
        ops.blockwise("sum", x, BLOCK, [3])
    assert e.value.status == 3
    with pytest.raises(XtgError) as e:
        ops.blockwise("sum", x, (5, 0, 2), [0])
    assert e.value.status == 1
