"""Evaluation entry points: assign (xt::noalias(out) = e), reductions
(xt::sum / mean / variance / amax / norm_l2 ... with axes, keep_dims,
initial, evaluation type T), arg-reductions (xt::argmax / argmin) and
accumulators (xt::cumsum / cumprod / nancumsum / nancumprod), index / filter /
masked views and .npy files (xt::load_npy / dump_npy)."""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Optional

import numpy as np

from ._ffi import ARG_MAX, ARG_MIN, RED, MAX_RANK, ReduceDesc, check, dtype_code, lib
from .device import DeviceArray, _sh
from .expr import as_expr, lower


def assign(out: DeviceArray, e, stream=None) -> DeviceArray:
    ex, keep = lower(as_expr(e))
    o = out.xtg_array()
    check(lib().xtg_assign(C.byref(ex), C.byref(o), _sh(stream)))
    return out


def broadcast_shape(e) -> tuple:
    ex, keep = lower(as_expr(e))
    r = C.c_int32()
    sh = (C.c_int64 * MAX_RANK)()
    check(lib().xtg_broadcast_shape(C.byref(ex), C.byref(r), sh))
    return tuple(sh[i] for i in range(r.value))


def expr_dtype(e) -> int:
    ex, keep = lower(as_expr(e))
    d = C.c_int32()
    check(lib().xtg_expr_dtype(C.byref(ex), C.byref(d)))
    return d.value


def make_desc(op: str, axes=None, keep_dims=False, initial=None, acc_dtype=None, ddof=0, precision=0) -> ReduceDesc:
    rd = ReduceDesc()
    rd.op = RED[op]
    if axes is None:
        rd.n_axes = -1
    else:
        if isinstance(axes, int):
            axes = [axes]
        axes = list(axes)
        rd.n_axes = len(axes)
        for i, a in enumerate(axes):
            rd.axes[i] = int(a)
    rd.keep_dims = 1 if keep_dims else 0
    rd.acc_dtype = -1 if acc_dtype is None else dtype_code(acc_dtype)
    rd.precision = precision
    rd.ddof = ddof
    if initial is not None:
        rd.has_initial = 1
        if isinstance(initial, float):
            rd.initial.f = initial
        else:
            rd.initial.i = int(initial)
    return rd


def reduce_shape(op: str, e, **kw):
    ex, keep = lower(as_expr(e))
    rd = make_desc(op, **kw)
    r = C.c_int32()
    sh = (C.c_int64 * MAX_RANK)()
    dt = C.c_int32()
    check(lib().xtg_reduce_shape(C.byref(ex), C.byref(rd), C.byref(r), sh, C.byref(dt)))
    return tuple(sh[i] for i in range(r.value)), dt.value


def reduce(op: str, e, axes=None, keep_dims=False, initial=None, acc_dtype=None, ddof=0, precision=0,
           out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """Evaluate a reducer into a new (or given) device array."""
    e = as_expr(e)
    kw = dict(axes=axes, keep_dims=keep_dims, initial=None, acc_dtype=acc_dtype, ddof=ddof, precision=precision)
    shape, dt = reduce_shape(op, e, **kw)
    if initial is not None:  # xt::initial(v) is converted to the result type
        from ._ffi import DTYPES
        initial = float(initial) if dt in (DTYPES["float32"], DTYPES["float64"], DTYPES["bfloat16"]) else int(initial)
    kw["initial"] = initial
    if out is None:
        out = DeviceArray.empty(shape, dt, stream)
    ex, keep = lower(e)
    rd = make_desc(op, **kw)
    o = out.xtg_array()
    check(lib().xtg_reduce(C.byref(ex), C.byref(rd), C.byref(o), _sh(stream)))
    return out


MOMENTS = ("sum", "mean", "variance", "norm_l2")


def reduce_moments(e, axes=None, keep_dims=False, ddof=0, which=MOMENTS, outs: Optional[dict] = None,
                   stream=None) -> dict:
    """sum, mean, variance (ddof) and norm_l2 of e over the same axes
    (xtg_reduce_moments: one pass over e when the plan streams, each result
    equal to its own reduce() call); returns {name: DeviceArray} for `which`."""
    e = as_expr(e)
    outs = dict(outs or {})
    for nm in which:
        if nm not in MOMENTS:
            raise ValueError(f"unknown moment {nm!r}")
        if nm not in outs:
            shape, dt = reduce_shape(nm, e, axes=axes, keep_dims=keep_dims, ddof=ddof if nm == "variance" else 0)
            outs[nm] = DeviceArray.empty(shape, dt, stream)
    ex, keep = lower(e)
    rd = make_desc("variance", axes=axes, keep_dims=keep_dims, ddof=ddof)
    arrs = [outs[nm].xtg_array() if nm in which else None for nm in MOMENTS]
    ptrs = [C.byref(a) if a is not None else None for a in arrs]
    check(lib().xtg_reduce_moments(C.byref(ex), C.byref(rd), *ptrs, _sh(stream)))
    return {nm: outs[nm] for nm in which}


def assign_reduce(out_e: DeviceArray, e, op: str, axes=None, keep_dims=False, initial=None, acc_dtype=None, ddof=0,
                  precision=0, out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """out_e = e, then the reduction `op` of out_e (xtg_assign_reduce: one
    pass when the plan allows); returns the reduction's result."""
    kw = dict(axes=axes, keep_dims=keep_dims, initial=None, acc_dtype=acc_dtype, ddof=ddof, precision=precision)
    shape, dt = reduce_shape(op, out_e, **kw)
    if initial is not None:
        from ._ffi import DTYPES
        initial = float(initial) if dt in (DTYPES["float32"], DTYPES["float64"], DTYPES["bfloat16"]) else int(initial)
    kw["initial"] = initial
    if out is None:
        out = DeviceArray.empty(shape, dt, stream)
    ex, keep = lower(as_expr(e))
    rd = make_desc(op, **kw)
    oe, o = out_e.xtg_array(), out.xtg_array()
    check(lib().xtg_assign_reduce(C.byref(ex), C.byref(oe), C.byref(rd), C.byref(o), _sh(stream)))
    return out


def argreduce(op: str, e, axis=None, out_dtype="int64", out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    from .ops import broadcast_shape as _bs
    e = as_expr(e)
    shape = _bs(e)
    if axis is None or len(shape) <= 1:
        oshape = ()
    else:
        a = axis + len(shape) if axis < 0 else axis
        oshape = tuple(n for i, n in enumerate(shape) if i != a)
    if out is None:
        out = DeviceArray.empty(oshape, out_dtype, stream)
    ex, keep = lower(e)
    o = out.xtg_array()
    code = ARG_MAX if op == "argmax" else ARG_MIN
    check(lib().xtg_argreduce(C.byref(ex), code, 0 if axis is None else 1, 0 if axis is None else int(axis),
                              C.byref(o), _sh(stream)))
    return out


def _red(name):
    def f(e, axes=None, **kw):
        return reduce(name, e, axes, **kw)
    f.__name__ = name
    return f


sum = _red("sum")  # noqa: A001
prod = _red("prod")
amax = _red("amax")
amin = _red("amin")
mean = _red("mean")
variance = _red("variance")
stddev = _red("stddev")
norm_l0 = _red("norm_l0")
norm_l1 = _red("norm_l1")
norm_sq = _red("norm_sq")
norm_l2 = _red("norm_l2")
norm_linf = _red("norm_linf")


def argmax(e, axis=None, **kw):
    return argreduce("argmax", e, axis, **kw)


def argmin(e, axis=None, **kw):
    return argreduce("argmin", e, axis, **kw)


ACC = {"cumsum": 0, "cumprod": 1, "nancumsum": 2, "nancumprod": 3}


def accumulate_shape(op: str, e, axis=None, acc_dtype=None):
    ex, keep = lower(as_expr(e))
    r = C.c_int32()
    sh = (C.c_int64 * MAX_RANK)()
    dt = C.c_int32()
    check(lib().xtg_accumulate_shape(C.byref(ex), ACC[op], 0 if axis is None else 1, 0 if axis is None else int(axis),
                                     -1 if acc_dtype is None else dtype_code(acc_dtype), C.byref(r), sh, C.byref(dt)))
    return tuple(sh[i] for i in range(r.value)), dt.value


def accumulate(op: str, e, axis=None, acc_dtype=None, out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """xt::cumsum / cumprod / nancumsum / nancumprod of `e` along `axis` (None:
    over the row-major flattening, a 1-D result); `acc_dtype` is the
    reference's template argument T."""
    e = as_expr(e)
    shape, dt = accumulate_shape(op, e, axis, acc_dtype)
    if out is None:
        out = DeviceArray.empty(shape, dt, stream)
    ex, keep = lower(e)
    o = out.xtg_array()
    check(lib().xtg_accumulate(C.byref(ex), ACC[op], 0 if axis is None else 1, 0 if axis is None else int(axis),
                               -1 if acc_dtype is None else dtype_code(acc_dtype), C.byref(o), _sh(stream)))
    return out


def cumsum(e, axis=None, **kw):
    return accumulate("cumsum", e, axis, **kw)


def cumprod(e, axis=None, **kw):
    return accumulate("cumprod", e, axis, **kw)


def nancumsum(e, axis=None, **kw):
    return accumulate("nancumsum", e, axis, **kw)


def nancumprod(e, axis=None, **kw):
    return accumulate("nancumprod", e, axis, **kw)


# ---- index, filter and masked views -------------------------------------------------------
SET_OPS = {"=": 0, "+=": 1, "-=": 2, "*=": 3, "/=": 4}


def _indices(indices, rank: int, stream=None) -> DeviceArray:
    import numpy as np
    if isinstance(indices, DeviceArray):
        return indices
    a = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1, rank))
    return DeviceArray.from_numpy(a, None, stream)


def index_view(e, indices, out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """Read xt::index_view(e, indices): out[k] = e[indices[k]] (indices: n
    coordinate rows of rank(e))."""
    e = as_expr(e)
    rank = len(broadcast_shape(e))
    idx = _indices(indices, rank, stream)
    n = idx.shape[0] if idx.ndim else 0
    if out is None:
        out = DeviceArray.empty((n,), expr_dtype(e), stream)
    ex, keep = lower(e)
    o = out.xtg_array()
    check(lib().xtg_gather(C.byref(ex), C.c_void_p(idx.ptr), n, C.byref(o), _sh(stream)))
    return out


def index_assign(dst: DeviceArray, indices, src, op: str = "=", stream=None) -> DeviceArray:
    """Assign through xt::index_view(dst, indices): dst[indices[k]] op= src[k]."""
    idx = _indices(indices, dst.ndim, stream)
    n = idx.shape[0]
    ex, keep = lower(as_expr(src))
    o = dst.xtg_array()
    check(lib().xtg_scatter(C.byref(ex), C.c_void_p(idx.ptr), n, SET_OPS[op], C.byref(o), _sh(stream)))
    return dst


def filter_count(cond, stream=None) -> int:
    ex, keep = lower(as_expr(cond))
    c = C.c_int64()
    check(lib().xtg_filter_count(C.byref(ex), C.byref(c), _sh(stream)))
    return c.value


def filter(e, cond, out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:  # noqa: A001
    """Read xt::filter(e, cond): the elements of e where cond holds, in
    row-major order (1-D)."""
    e, cond = as_expr(e), as_expr(cond)
    if out is None:
        out = DeviceArray.empty((filter_count(cond, stream),), expr_dtype(e), stream)
    ex, k1 = lower(e)
    cx, k2 = lower(cond)
    o = out.xtg_array()
    check(lib().xtg_filter(C.byref(ex), C.byref(cx), C.byref(o), _sh(stream)))
    return out


def filter_assign(dst: DeviceArray, cond, src, op: str = "=", stream=None) -> DeviceArray:
    """Assign through xt::filter(dst, cond) (src 1-D of the selected count)
    or xt::filtration(dst, cond) (src a scalar)."""
    sx, k1 = lower(as_expr(src))
    cx, k2 = lower(as_expr(cond))
    o = dst.xtg_array()
    check(lib().xtg_filter_assign(C.byref(sx), C.byref(cx), SET_OPS[op], C.byref(o), _sh(stream)))
    return dst


def masked_assign(dst: DeviceArray, mask, src, op: str = "=", stream=None) -> DeviceArray:
    """Assign through xt::masked_view(dst, mask): where mask holds,
    dst op= src (src and mask broadcast to dst)."""
    sx, k1 = lower(as_expr(src))
    mx, k2 = lower(as_expr(mask))
    o = dst.xtg_array()
    check(lib().xtg_masked_assign(C.byref(sx), C.byref(mx), SET_OPS[op], C.byref(o), _sh(stream)))
    return dst


# ---- .npy files (xt::load_npy / xt::dump_npy, io/xnpy.hpp) ----------------------------

def _npy_source(src):
    """(path bytes, None) for a file name, (None, buffer) for a file image."""
    import os
    if isinstance(src, (str, os.PathLike)):
        return os.fsencode(src), None
    mv = memoryview(src)
    if not mv.c_contiguous:
        raise ValueError("npy buffer must be contiguous")
    return None, mv.cast("B")


def npy_header(src) -> dict:
    """The header of a .npy file (path) or file image (bytes-like)."""
    from ._ffi import NpyHeader
    h = NpyHeader()
    path, mv = _npy_source(src)
    if path is not None:
        check(lib().xtg_npy_info(path, C.byref(h)))
    else:
        a = np.frombuffer(mv, dtype=np.uint8)  # no copy of the image
        check(lib().xtg_npy_info_buffer(a.ctypes.data, a.nbytes, C.byref(h)))
    return {"descr": h.descr.decode(), "dtype": h.dtype, "fortran_order": bool(h.fortran_order),
            "version": h.version, "shape": tuple(h.shape[i] for i in range(h.rank)),
            "data_offset": h.data_offset, "data_bytes": h.data_bytes}


def load_npy(src, dtype=None, layout: str = "dynamic", out: Optional[DeviceArray] = None,
             stream=None) -> DeviceArray:
    """xt::load_npy<T, L>(filename) / load_npy<T, L>(std::istream&) into
    device memory.  ``src`` is a path or a bytes-like file image; ``dtype`` is
    T (default: the file's own type); ``layout`` is L ("dynamic",
    "row_major", "column_major").  A Fortran-order file loads into a
    column-major array, as the reference's dynamic-layout result."""
    from ._ffi import LAYOUTS, XtgError
    h = npy_header(src)
    if out is None:
        if dtype is None:
            if h["dtype"] < 0:
                raise XtgError(1, f"Cast error: formats not matching {h['descr']} vs (no device type)")
            code = h["dtype"]
        else:
            code = dtype_code(dtype)
        shape = h["shape"]
        n = int(np.prod(shape)) if shape else 1
        buf = DeviceArray.empty((n,), code, stream)
        if h["fortran_order"]:
            st, acc = [], 1
            for d in shape:
                st.append(acc)
                acc *= max(int(d), 1)
            out = DeviceArray(shape, code, buf.ptr, st, base=buf)
        else:
            out = DeviceArray(shape, code, buf.ptr, base=buf)
    o = out.xtg_array()
    path, mv = _npy_source(src)
    if path is not None:
        check(lib().xtg_npy_load(path, C.byref(o), LAYOUTS[layout], _sh(stream)))
    else:
        a = np.frombuffer(mv, dtype=np.uint8)
        check(lib().xtg_npy_load_buffer(a.ctypes.data, a.nbytes, C.byref(o), LAYOUTS[layout], _sh(stream)))
    return out


def _npy_device_source(e, stream):
    if isinstance(e, DeviceArray):
        return e
    from .expr import as_expr
    ex = as_expr(e)
    t = DeviceArray.empty(broadcast_shape(ex), expr_dtype(ex), stream)
    return assign(t, ex, stream)


def dump_npy(*args, stream=None):
    """xt::dump_npy(filename, e) writes a file; xt::dump_npy(e) returns the
    file image as bytes.  ``e`` is a device array or an expression (evaluated
    first, as the reference's eval)."""
    import os
    # `src` holds an evaluated temporary alive until the bytes are out
    if len(args) == 2:
        path, e = args
        src = _npy_device_source(e, stream)
        a = src.xtg_array()
        check(lib().xtg_npy_save(os.fsencode(path), C.byref(a), _sh(stream)))
        return None
    (e,) = args
    src = _npy_device_source(e, stream)
    a = src.xtg_array()
    n = C.c_size_t()
    check(lib().xtg_npy_save_buffer(C.byref(a), None, 0, C.byref(n), _sh(stream)))
    out = bytearray(n.value)
    buf = (C.c_char * n.value).from_buffer(out)
    check(lib().xtg_npy_save_buffer(C.byref(a), buf, n.value, C.byref(n), _sh(stream)))
    return bytes(out)


def npy_format_header(dtype, shape, fortran_order: bool = False) -> bytes:
    """The header bytes dump_npy writes before the data (host only)."""
    shp = (C.c_int64 * MAX_RANK)(*[int(s) for s in shape])
    n = C.c_size_t()
    code = dtype_code(dtype)
    check(lib().xtg_npy_format_header(code, int(fortran_order), len(shape), shp, None, 0, C.byref(n)))
    out = bytearray(n.value)
    buf = (C.c_char * n.value).from_buffer(out)
    check(lib().xtg_npy_format_header(code, int(fortran_order), len(shape), shp, buf, n.value, C.byref(n)))
    return bytes(out)


# ---- blockwise reducers (xt::blockwise::*, reducers/xblockwise_reducer.hpp) -----------

def _blockwise_array(x):
    """(xtg_array, keepalive) for a device array or a host numpy array."""
    from .device import HostArray
    if isinstance(x, DeviceArray):
        return x.xtg_array(), x
    if isinstance(x, np.ndarray):
        h = HostArray(x)
        return h.xtg_array(), h
    raise TypeError("blockwise input must be a DeviceArray or a host numpy array")


def blockwise_shape(op: str, x, axes=None, keep_dims=False, acc_dtype=None):
    a, keep = _blockwise_array(x)
    rd = make_desc(op, axes, keep_dims, acc_dtype=acc_dtype)
    r = C.c_int32()
    sh = (C.c_int64 * MAX_RANK)()
    dt = C.c_int32()
    check(lib().xtg_blockwise_shape(C.byref(a), C.byref(rd), C.byref(r), sh, C.byref(dt)))
    return tuple(sh[i] for i in range(r.value)), dt.value


def blockwise(op: str, x, block_shape, axes=None, keep_dims=False, p: float = 2.0, acc_dtype=None,
              out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """xt::blockwise::<op>(x, block_shape, axes, options) evaluated into a
    device array (``reducer.assign_to(result)``).  ``x`` is a device array or
    a host numpy array (pageable or pinned; it may be larger than device
    memory: it streams through in slabs of whole blocks).  ``p`` is the
    exponent of norm_lp_to_p / norm_lp."""
    a, keep = _blockwise_array(x)
    rd = make_desc(op, axes, keep_dims, acc_dtype=acc_dtype)
    if out is None:
        shape, dt = blockwise_shape(op, x, axes, keep_dims, acc_dtype)
        out = DeviceArray.empty(shape, dt, stream)
    bs = (C.c_int64 * MAX_RANK)(*[int(b) for b in block_shape])
    if len(block_shape) != len(a.shape[:a.rank]):
        raise ValueError("block_shape must have one extent per dimension")
    o = out.xtg_array()
    check(lib().xtg_blockwise_reduce(C.byref(a), bs, C.byref(rd), float(p), C.byref(o), _sh(stream)))
    return out
