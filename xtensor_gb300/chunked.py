"""Chunked arrays in device memory: xt::xchunked_array / xt::chunked_array
(include/xtensor/chunk/xchunked_array.hpp:56-686) and xt::as_chunked
(chunk/xchunked_view.hpp), over the C ABI's xtg_chunked_* entry points.

A ChunkedArray cuts its shape into a grid of ceil(shape / chunk_shape)
chunks, each a device buffer of chunk_shape elements (one allocation holds
them all, at equal distances); the last chunk along a dimension ends inside
its buffer (padding), as in the reference.  It
is an expression leaf like DeviceArray, so `a.assign(a + a)`, `a += 2.0`,
`a.assign(b * 3)` and reductions work on it; chunked operands of one
assignment must share the destination's grid.
"""
from __future__ import annotations

import ctypes as C
import itertools
import math
from typing import Optional, Sequence

import numpy as np

from ._ffi import MAX_RANK, Array, ReduceDesc, check, dtype_code, lib, np_dtype, ITEMSIZE
from .device import D2H, H2D, DeviceArray, _sh
from .expr import ExprOps, as_expr, lower


class Chunked(C.Structure):
    _fields_ = [("chunks", C.c_void_p), ("dtype", C.c_int32), ("rank", C.c_int32),
                ("shape", C.c_int64 * MAX_RANK), ("chunk_shape", C.c_int64 * MAX_RANK)]


_SIGS_DONE = [False]


def _sigs():
    if _SIGS_DONE[0]:
        return lib()
    L = lib()
    P, vp, st = C.POINTER, C.c_void_p, C.c_int
    L.xtg_chunked_assign.argtypes = [vp, vp, P(Chunked), vp]
    L.xtg_chunked_assign.restype = st
    L.xtg_chunked_to_dense.argtypes = [P(Chunked), P(Array), vp]
    L.xtg_chunked_to_dense.restype = st
    L.xtg_chunked_reduce.argtypes = [P(Chunked), P(ReduceDesc), P(Array), vp]
    L.xtg_chunked_reduce.restype = st
    _SIGS_DONE[0] = True
    return L


def grid_shape(shape: Sequence[int], chunk_shape: Sequence[int]) -> tuple:
    """Chunks per dimension, the edge chunk included (xchunked_array.hpp:601-616)."""
    return tuple(s // c + (1 if s % c else 0) for s, c in zip(shape, chunk_shape))


class ChunkedArray(ExprOps):
    """A chunked array of `shape` in chunks of `chunk_shape` (each chunk a
    device buffer of chunk_shape elements, row-major)."""

    def __init__(self, shape, chunk_shape, dtype, stream=None, chunks=None):
        self.shape = tuple(int(s) for s in shape)
        self.chunk_shape = tuple(int(c) for c in chunk_shape)
        if len(self.chunk_shape) != len(self.shape):
            raise ValueError("chunk shape and shape must have the same rank")
        if any(c < 1 for c in self.chunk_shape):
            raise ValueError("chunk extents must be positive")
        self.dtype = dtype_code(dtype)
        self.grid_shape = grid_shape(self.shape, self.chunk_shape)
        n = math.prod(self.grid_shape)
        if chunks is None:
            # one slab, chunks at a fixed 256-byte aligned distance: the
            # library then reduces a class of equal chunks as one strided array
            es = ITEMSIZE[self.dtype]
            dist = -(-max(math.prod(self.chunk_shape) * es, 1) // 256) * 256
            self._slab = DeviceArray.empty((n * dist // es,), self.dtype, stream)
            chunks = [DeviceArray(self.chunk_shape, self.dtype, self._slab.ptr + i * dist, base=self._slab)
                      for i in range(n)]
        self.chunks = list(chunks)
        if len(self.chunks) != n:
            raise ValueError("one chunk per grid cell")
        self._ptrs = (C.c_void_p * max(n, 1))(*[c.ptr for c in self.chunks])

    # ---- construction helpers (xt::chunked_array overloads, :262-345)
    @classmethod
    def from_expr(cls, e, chunk_shape=None, stream=None) -> "ChunkedArray":
        """chunked_array(e, chunk_shape): a new chunked array assigned from e;
        without a chunk shape, a chunked e gives its own, any other e its
        shape (one chunk)."""
        from .ops import broadcast_shape, expr_dtype
        if isinstance(e, ChunkedArray):
            shape, dt = e.shape, e.dtype
            chunk_shape = e.chunk_shape if chunk_shape is None else chunk_shape
        else:
            shape, dt = broadcast_shape(e), expr_dtype(e)
            chunk_shape = shape if chunk_shape is None else chunk_shape
        a = cls(shape, chunk_shape, dt, stream)
        a.assign(e, stream)
        return a

    @classmethod
    def from_numpy(cls, x: np.ndarray, chunk_shape, dtype=None, stream=None) -> "ChunkedArray":
        return cls.from_expr(DeviceArray.from_numpy(x, dtype, stream), chunk_shape, stream)

    # ---- descriptors
    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def size(self) -> int:
        return math.prod(self.shape)

    @property
    def grid_size(self) -> int:
        return len(self.chunks)

    def xtg_chunked(self) -> Chunked:
        c = Chunked()
        c.chunks = C.cast(self._ptrs, C.c_void_p).value
        c.dtype = self.dtype
        c.rank = self.ndim
        for d in range(self.ndim):
            c.shape[d] = self.shape[d]
            c.chunk_shape[d] = self.chunk_shape[d]
        return c

    def xtg_array(self) -> Array:
        """Stand-in leaf descriptor (dtype and shape; the library takes the
        data from the chunk table)."""
        a = Array()
        a.data = self.chunks[0].ptr if self.chunks else 1
        a.dtype = self.dtype
        a.rank = self.ndim
        s = 1
        for d in range(self.ndim - 1, -1, -1):
            a.shape[d] = self.shape[d]
            a.strides[d] = s
            s *= max(self.shape[d], 1)
        return a

    # ---- element access (operator(), xchunked_array.hpp:440-460)
    def _locate(self, idx):
        if len(idx) != self.ndim:
            raise IndexError("one index per dimension")
        ci, off = 0, 0
        cst = [1] * self.ndim
        for d in range(self.ndim - 2, -1, -1):
            cst[d] = cst[d + 1] * self.chunk_shape[d + 1]
        for d, i in enumerate(idx):
            i = int(i)
            if not 0 <= i < self.shape[d]:
                raise IndexError("index out of range")
            ci = ci * self.grid_shape[d] + i // self.chunk_shape[d]
            off += (i % self.chunk_shape[d]) * cst[d]
        return self.chunks[ci].ptr + off * ITEMSIZE[self.dtype]

    def __getitem__(self, idx):
        idx = idx if isinstance(idx, tuple) else (idx,)
        v = np.zeros((), np_dtype(self.dtype))
        check(lib().xtg_memcpy(v.ctypes.data, self._locate(idx), v.nbytes, D2H, None))
        return v[()]

    def __setitem__(self, idx, value):
        idx = idx if isinstance(idx, tuple) else (idx,)
        v = np.asarray(value, dtype=np_dtype(self.dtype))
        check(lib().xtg_memcpy(self._locate(idx), v.ctypes.data, v.nbytes, H2D, None))
        check(lib().xtg_device_sync())

    # ---- chunks (chunk_begin / xchunk_iterator, xchunked_assign.hpp:236-372)
    def chunk_items(self):
        """(chunk index, chunk buffer, region slices) in the grid's row-major order."""
        for ci, gc in enumerate(itertools.product(*[range(g) for g in self.grid_shape])):
            sl = tuple(slice(g * c, min((g + 1) * c, s)) for g, c, s in zip(gc, self.chunk_shape, self.shape))
            yield gc, self.chunks[ci], sl

    # ---- evaluation
    def assign(self, e, stream=None) -> "ChunkedArray":
        """self = e, chunk by chunk (noalias(a) = e / a = e)."""
        return chunked_assign(self, e, stream)

    def _computed(self, op, o):
        return self.assign(op(self._e(), o))

    def __iadd__(self, o): return self._computed(lambda a, b: a + b, o)
    def __isub__(self, o): return self._computed(lambda a, b: a - b, o)
    def __imul__(self, o): return self._computed(lambda a, b: a * b, o)
    def __itruediv__(self, o): return self._computed(lambda a, b: a / b, o)

    def to_device(self, out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
        """A dense device array with the chunked array's values."""
        if out is None:
            out = DeviceArray.empty(self.shape, self.dtype, stream)
        o = out.xtg_array()
        c = self.xtg_chunked()
        check(_sigs().xtg_chunked_to_dense(C.byref(c), C.byref(o), _sh(stream)))
        return out

    def to_numpy(self, stream=None) -> np.ndarray:
        return self.to_device(stream=stream).to_numpy(stream)


def chunked_assign(dst: ChunkedArray, e, stream=None) -> ChunkedArray:
    ex, leaves = lower(as_expr(e))
    cl = (C.c_void_p * max(len(leaves), 1))()
    keep = []
    for i, lf in enumerate(leaves):
        if isinstance(lf, ChunkedArray):
            c = lf.xtg_chunked()
            keep.append(c)
            cl[i] = C.addressof(c)
    d = dst.xtg_chunked()
    check(_sigs().xtg_chunked_assign(C.addressof(ex), C.addressof(cl), C.byref(d), _sh(stream)))
    return dst


def as_chunked_assign(dst: DeviceArray, chunk_shape, e, stream=None) -> DeviceArray:
    """as_chunked(dst, chunk_shape) = e: the chunk-by-chunk assignment of a
    chunked view over a dense array.  A chunked source is read with its own
    grid; any other expression is one assignment (the values are the same
    in whatever order the chunks are walked)."""
    if isinstance(e, ChunkedArray):
        return e.to_device(dst, stream)
    from .ops import assign
    return assign(dst, e, stream)


def chunked_reduce(op: str, src: ChunkedArray, axes=None, keep_dims=False, acc_dtype=None,
                   out: Optional[DeviceArray] = None, stream=None) -> DeviceArray:
    """A reducer over a chunked array (xt::sum(a, axes), ...): one strided
    reduction per class of equal chunks when the chunks sit at equal
    distances (as this module allocates them), chunk by chunk otherwise."""
    from .ops import make_desc, reduce_shape
    shape, dt = reduce_shape(op, _DenseLike(src), axes=axes, keep_dims=keep_dims, acc_dtype=acc_dtype)
    if out is None:
        out = DeviceArray.empty(shape, dt, stream)
    rd = make_desc(op, axes=axes, keep_dims=keep_dims, acc_dtype=acc_dtype)
    c = src.xtg_chunked()
    o = out.xtg_array()
    check(_sigs().xtg_chunked_reduce(C.byref(c), C.byref(rd), C.byref(o), _sh(stream)))
    return out


class _DenseLike(ExprOps):
    """Shape-and-type stand-in of a chunked array for shape queries."""

    def __init__(self, src: ChunkedArray):
        self.src, self.dtype, self.shape = src, src.dtype, src.shape

    def xtg_array(self) -> Array:
        return self.src.xtg_array()
