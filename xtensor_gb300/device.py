"""Device arrays and streams over libxtg's allocation / copy entry points."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from ._ffi import ITEMSIZE, MAX_RANK, Array, check, dtype_code, lib, np_dtype
from .expr import ExprOps

H2D, D2H, D2D = 1, 2, 3


def init(device: int = -1) -> None:
    check(lib().xtg_init(device))


def device_sync() -> None:
    check(lib().xtg_device_sync())


class Stream:
    """A non-blocking CUDA stream created by libxtg."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().xtg_stream_create(C.byref(h)))
        self.handle = h.value

    def sync(self) -> None:
        check(lib().xtg_stream_sync(self.handle))

    def close(self) -> None:
        if self.handle:
            lib().xtg_stream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _sh(stream):
    if stream is None:
        return None
    return stream.handle if isinstance(stream, Stream) else stream


class _Buffer:
    def __init__(self, nbytes: int, stream=None):
        p = C.c_void_p()
        check(lib().xtg_malloc(C.byref(p), max(int(nbytes), 1), _sh(stream)))
        self.ptr = p.value
        self.nbytes = nbytes

    def __del__(self):
        try:
            if self.ptr:
                lib().xtg_free(self.ptr, None)
        except Exception:
            pass


def contiguous_strides(shape: Sequence[int]) -> tuple[int, ...]:
    st = []
    acc = 1
    for n in reversed(shape):
        st.append(acc)
        acc *= max(int(n), 1)
    return tuple(reversed(st))


class DeviceArray(ExprOps):
    """A strided array in device memory (strides in elements, like xtensor)."""

    def __init__(self, shape, dtype, ptr: int, strides=None, base=None):
        self.shape = tuple(int(s) for s in shape)
        self.dtype = dtype_code(dtype)
        self.ptr = int(ptr) if ptr else 0
        self.strides = tuple(strides) if strides is not None else contiguous_strides(self.shape)
        self.base = base
        if len(self.shape) > MAX_RANK:
            raise ValueError("rank > 8")

    # construction
    @classmethod
    def empty(cls, shape, dtype, stream=None) -> "DeviceArray":
        shape = tuple(int(s) for s in shape)
        n = int(np.prod(shape)) if shape else 1
        buf = _Buffer(n * ITEMSIZE[dtype_code(dtype)], stream)
        return cls(shape, dtype, buf.ptr, base=buf)

    @classmethod
    def from_numpy(cls, a: np.ndarray, dtype=None, stream=None) -> "DeviceArray":
        code = dtype_code(dtype if dtype is not None else a.dtype)
        a = np.ascontiguousarray(a)
        d = cls.empty(a.shape, code, stream)
        if a.nbytes:
            check(lib().xtg_memcpy(d.ptr, a.ctypes.data, a.nbytes, H2D, _sh(stream)))
            check(lib().xtg_stream_sync(_sh(stream)))
        return d

    # properties
    @property
    def size(self) -> int:
        return int(np.prod(self.shape)) if self.shape else 1

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def itemsize(self) -> int:
        return ITEMSIZE[self.dtype]

    @property
    def nbytes(self) -> int:
        return self.size * self.itemsize

    def is_contiguous(self) -> bool:
        return self.strides == contiguous_strides(self.shape) or self.size <= 1

    def xtg_array(self) -> Array:
        a = Array()
        a.data = self.ptr
        a.dtype = self.dtype
        a.rank = len(self.shape)
        for i, (n, s) in enumerate(zip(self.shape, self.strides)):
            a.shape[i] = n
            a.strides[i] = s
        return a

    # views (strided_view / transpose: no copy)
    def transpose(self, perm=None) -> "DeviceArray":
        perm = tuple(range(self.ndim))[::-1] if perm is None else tuple(perm)
        return DeviceArray([self.shape[p] for p in perm], self.dtype, self.ptr,
                           [self.strides[p] for p in perm], base=self)

    def reshape(self, shape) -> "DeviceArray":
        if not self.is_contiguous():
            raise ValueError("reshape of a non-contiguous view")
        shape = tuple(int(s) for s in shape)
        if int(np.prod(shape)) != self.size:
            raise ValueError("reshape size mismatch")
        return DeviceArray(shape, self.dtype, self.ptr, base=self)

    def __getitem__(self, key) -> "DeviceArray":
        if not isinstance(key, tuple):
            key = (key,)
        shape, strides, off = [], [], 0
        dims = list(zip(self.shape, self.strides))
        ki = 0
        for d, (n, s) in enumerate(dims):
            k = key[ki] if ki < len(key) else slice(None)
            ki += 1
            if isinstance(k, slice):
                start, stop, step = k.indices(n)
                cnt = len(range(start, stop, step))
                off += start * s
                shape.append(cnt)
                strides.append(s * step)
            else:
                k = int(k)
                if k < 0:
                    k += n
                if not 0 <= k < n:
                    raise IndexError("index out of range")
                off += k * s
        return DeviceArray(shape, self.dtype, self.ptr + off * self.itemsize, strides, base=self)

    # copies
    def to_numpy(self, stream=None) -> np.ndarray:
        src = self
        if not self.is_contiguous():
            from .ops import assign
            from .expr import leaf
            src = DeviceArray.empty(self.shape, self.dtype, stream)
            assign(src, leaf(self), stream=stream)
        out = np.empty(self.shape, dtype=np_dtype(self.dtype))
        if out.nbytes:
            check(lib().xtg_memcpy(out.ctypes.data, src.ptr, out.nbytes, D2H, _sh(stream)))
        check(lib().xtg_stream_sync(_sh(stream)))
        return out

    def copy_from(self, a: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes == self.nbytes and self.is_contiguous()
        check(lib().xtg_memcpy(self.ptr, a.ctypes.data, a.nbytes, H2D, _sh(stream)))

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype}, strides={self.strides})"


class HostArray(ExprOps):
    """A numpy array exposed as an ``xtg_array`` with a host pointer (used by
    the oracle and by dry-run planning)."""

    def __init__(self, a: np.ndarray, dtype=None):
        self.a = a
        self.dtype = dtype_code(dtype if dtype is not None else a.dtype)
        self.shape = a.shape
        self.strides = tuple(s // a.itemsize for s in a.strides)

    def xtg_array(self) -> Array:
        x = Array()
        x.data = self.a.ctypes.data if self.a.size else 1
        x.dtype = self.dtype
        x.rank = self.a.ndim
        for i in range(self.a.ndim):
            x.shape[i] = self.a.shape[i]
            x.strides[i] = self.strides[i]
        return x
