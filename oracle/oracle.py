"""ctypes binding of the C oracle (xt_oracle.c) — test infrastructure only.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module; the product path never does.  Inputs are host
numpy arrays wrapped as ``xtg_array`` (HostArray); expressions are the same
lowered ``xtg_expr`` the GPU library takes.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from xtensor_gb300._ffi import MAX_RANK, Array, Expr, ReduceDesc, dtype_code, np_dtype
from xtensor_gb300.device import HostArray
from xtensor_gb300.expr import as_expr, lower
from xtensor_gb300.ops import make_desc

SO = Path(__file__).resolve().parent / "_build" / "liboracle.so"
_L = None


def lib():
    global _L
    if _L is None:
        if not SO.exists():
            from xtensor_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(SO))
        P = C.POINTER
        L.orc_assign.argtypes = [P(Expr), P(Array)]
        L.orc_reduce.argtypes = [P(Expr), P(ReduceDesc), P(Array)]
        L.orc_argreduce.argtypes = [P(Expr), C.c_int, C.c_int, C.c_int64, P(Array)]
        L.orc_expr_dtype.argtypes = [P(Expr)]
        L.orc_broadcast_shape.argtypes = [P(Expr), P(C.c_int32), P(C.c_int64)]
        L.orc_reduce_result_dtype.argtypes = [P(Expr), P(ReduceDesc)]
        L.orc_last_error.restype = C.c_char_p
        L.orc_promote.argtypes = [C.c_int, C.c_int]
        L.orc_accumulate_dtype.argtypes = [P(Expr), C.c_int, C.c_int]
        L.orc_accumulate.argtypes = [P(Expr), C.c_int, C.c_int, C.c_int64, C.c_int, P(Array)]
        _L = L
    return _L


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle status {code}: {msg}")
        self.status = code


def _chk(s):
    if s != 0:
        raise OracleError(s, lib().orc_last_error().decode())


def host(a: np.ndarray, dtype=None) -> HostArray:
    return HostArray(a, dtype)


def expr_dtype(e) -> int:
    ex, keep = lower(as_expr(e))
    return lib().orc_expr_dtype(C.byref(ex))


def broadcast_shape(e):
    ex, keep = lower(as_expr(e))
    r = C.c_int32()
    sh = (C.c_int64 * MAX_RANK)()
    _chk(lib().orc_broadcast_shape(C.byref(ex), C.byref(r), sh))
    return tuple(sh[i] for i in range(r.value))


def assign(e, shape=None, dtype=None) -> np.ndarray:
    """Evaluate `e` (over HostArray leaves) into a new numpy array."""
    e = as_expr(e)
    shape = broadcast_shape(e) if shape is None else tuple(shape)
    code = expr_dtype(e) if dtype is None else dtype_code(dtype)
    out = np.zeros(shape, dtype=np_dtype(code))
    ho = HostArray(out, code)
    ex, keep = lower(e)
    o = ho.xtg_array()
    _chk(lib().orc_assign(C.byref(ex), C.byref(o)))
    return out


def reduce(op, e, axes=None, keep_dims=False, initial=None, acc_dtype=None, ddof=0) -> np.ndarray:
    e = as_expr(e)
    rd = make_desc(op, axes=axes, keep_dims=keep_dims, initial=initial, acc_dtype=acc_dtype, ddof=ddof)
    ex, keep = lower(e)
    code = lib().orc_reduce_result_dtype(C.byref(ex), C.byref(rd))
    shape = broadcast_shape(e)
    rank = len(shape)
    if axes is None:
        ax = list(range(rank))
    else:
        ax = [a + rank if a < 0 else a for a in ([axes] if isinstance(axes, int) else list(axes))]
    oshape = tuple((1 if i in ax else n) for i, n in enumerate(shape) if keep_dims or i not in ax)
    out = np.zeros(oshape, dtype=np_dtype(code))
    ho = HostArray(out, code)
    o = ho.xtg_array()
    _chk(lib().orc_reduce(C.byref(ex), C.byref(rd), C.byref(o)))
    return out


def argreduce(op, e, axis=None) -> np.ndarray:
    e = as_expr(e)
    shape = broadcast_shape(e)
    if axis is None or len(shape) <= 1:
        oshape = ()
    else:
        a = axis + len(shape) if axis < 0 else axis
        oshape = tuple(n for i, n in enumerate(shape) if i != a)
    out = np.zeros(oshape, dtype=np.int64)
    ho = HostArray(out)
    ex, keep = lower(e)
    o = ho.xtg_array()
    code = 0 if op == "argmax" else 1
    _chk(lib().orc_argreduce(C.byref(ex), code, 0 if axis is None else 1, 0 if axis is None else axis, C.byref(o)))
    return out


ACC_OPS = {"cumsum": 0, "cumprod": 1, "nancumsum": 2, "nancumprod": 3}


def accumulate(op, e, axis=None, acc_dtype=None) -> np.ndarray:
    """xt::cumsum / cumprod / nancumsum / nancumprod of `e` over `axis` (None:
    the row-major flattening, a 1-D result)."""
    e = as_expr(e)
    ex, keep = lower(e)
    code = ACC_OPS[op]
    acc = -1 if acc_dtype is None else dtype_code(acc_dtype)
    dt = lib().orc_accumulate_dtype(C.byref(ex), code, acc)
    if dt < 0:
        _chk(-dt)
    shape = broadcast_shape(e)
    oshape = (int(np.prod(shape, dtype=np.int64)),) if axis is None else shape
    out = np.zeros(oshape, dtype=np_dtype(dt))
    ho = HostArray(out, dt)
    o = ho.xtg_array()
    _chk(lib().orc_accumulate(C.byref(ex), code, 0 if axis is None else 1, 0 if axis is None else int(axis), acc,
                              C.byref(o)))
    return out


# ---- index, filter and masked views ---------------------------------------------------------
# Restatements of the reference's view semantics, over values the C oracle
# evaluates (orc_assign), with the C++ conversions of `dst op= value`
# (computed in the promoted type, stored as the destination type):
#  * index_view read: v(i) = e[indices[i]] (include/xtensor/views/xindex_view.hpp:398-488);
#  * index_view assignment: element by element in index order through the
#    view's stepper (xview_semantic), so a repeated coordinate is written
#    once per occurrence, in order;
#  * filter(e, cond) = index_view(e, argwhere(cond)), argwhere in row-major
#    order (xindex_view.hpp:821-826); filtration(e, cond) op= scalar applies
#    `cond ? op(e, scalar) : e` element by element (:763-767);
#  * masked_view(dst, mask) = e copies e through the view's iterator, which
#    skips masked elements (include/xtensor/views/xmasked_view.hpp:577-594).
def _set_apply(op, a, b, ct, dt):
    a = a.astype(ct)
    b = np.asarray(b).astype(ct)
    if op == "=":
        r = b
    elif op == "+=":
        r = a + b
    elif op == "-=":
        r = a - b
    elif op == "*=":
        r = a * b
    elif np.issubdtype(ct, np.floating):
        r = a / b
    else:
        # C++ integer division truncates toward zero
        bb = np.where(b == 0, 1, b)
        q = np.abs(a) // np.abs(bb)
        r = np.where(b != 0, np.where((a < 0) != (bb < 0), -q, q), 0).astype(ct)
    return r.astype(dt)


def index_view(e, indices) -> np.ndarray:
    v = assign(e)
    idx = np.asarray(indices, dtype=np.int64).reshape(-1, v.ndim)
    return np.array([v[tuple(ix)] for ix in idx], dtype=v.dtype)


def index_assign(dst: np.ndarray, indices, src, op="=") -> np.ndarray:
    """dst (numpy, modified and returned) through index_view(dst, indices)."""
    idx = np.asarray(indices, dtype=np.int64).reshape(-1, dst.ndim)
    s = assign(src) if not np.isscalar(src) else np.asarray(src)
    s = np.broadcast_to(s, (len(idx),))
    ct = np_dtype(lib().orc_promote(dtype_code(dst.dtype), dtype_code(s.dtype)))
    for k, ix in enumerate(idx):
        dst[tuple(ix)] = _set_apply(op, np.asarray(dst[tuple(ix)]), s[k], ct, dst.dtype)
    return dst


def filter(e, cond) -> np.ndarray:  # noqa: A001
    v = assign(e)
    c = assign(cond).astype(bool)
    return np.array([v[tuple(ix)] for ix in np.argwhere(c)], dtype=v.dtype)


def filter_assign(dst: np.ndarray, cond, src, op="=") -> np.ndarray:
    c = assign(cond).astype(bool)
    pos = np.argwhere(c)
    s = assign(src) if not np.isscalar(src) else np.asarray(src)
    s = np.broadcast_to(s, (len(pos),))
    ct = np_dtype(lib().orc_promote(dtype_code(dst.dtype), dtype_code(s.dtype)))
    for k, ix in enumerate(pos):
        dst[tuple(ix)] = _set_apply(op, np.asarray(dst[tuple(ix)]), s[k], ct, dst.dtype)
    return dst


def masked_assign(dst: np.ndarray, mask, src, op="=") -> np.ndarray:
    m = np.broadcast_to(assign(mask).astype(bool), dst.shape)
    s = np.broadcast_to(assign(src) if not np.isscalar(src) else np.asarray(src), dst.shape)
    ct = np_dtype(lib().orc_promote(dtype_code(dst.dtype), dtype_code(s.dtype)))
    for ix in np.argwhere(m):
        dst[tuple(ix)] = _set_apply(op, np.asarray(dst[tuple(ix)]), s[tuple(ix)], ct, dst.dtype)
    return dst
