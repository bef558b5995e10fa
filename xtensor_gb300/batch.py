"""Batched evaluation of many instances of one expression shape
(xtg_batch_*): one persistent launch, optional CUDA-graph replay, measured
autotuning.

    b = Batch(A0 * v0 + C0, reduce="sum")         # template: first instance
    for A, v, C, r in instances:
        b.add(A * v + C, r)                          # same tree shape
    b.build(autotune=True)
    b.run()            # or: b.capture(stream); b.replay(stream)
"""
from __future__ import annotations

import ctypes as C

from ._ffi import Array, Expr, ReduceDesc, check, lib
from .device import Stream, _sh
from .expr import as_expr, lower
from .ops import make_desc


class BatchInfo(C.Structure):
    _fields_ = [("instances", C.c_int64), ("tiles", C.c_int64), ("elements", C.c_int64),
                ("algorithmic_bytes", C.c_int64), ("group_lanes", C.c_int32), ("unroll", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("tuned", C.c_int32), ("tile_elems", C.c_int64),
                ("graph_ready", C.c_int32), ("pad", C.c_int32)]


def _sigs(L):
    P, vp, i32 = C.POINTER, C.c_void_p, C.c_int32
    L.xtg_batch_create.argtypes = [P(Expr), P(ReduceDesc), P(vp)]
    L.xtg_batch_add.argtypes = [vp, P(Array), i32, P(Array)]
    L.xtg_batch_build.argtypes = [vp, i32, vp]
    L.xtg_batch_run.argtypes = [vp, vp]
    L.xtg_batch_capture.argtypes = [vp, vp]
    L.xtg_batch_replay.argtypes = [vp, vp]
    L.xtg_batch_get_info.argtypes = [vp, P(BatchInfo)]
    L.xtg_batch_destroy.argtypes = [vp]
    L.xtg_fill_random.argtypes = [P(Array), i32, C.c_double, C.c_double, C.c_uint64, vp]
    for n in ("xtg_batch_create", "xtg_batch_add", "xtg_batch_build", "xtg_batch_run", "xtg_batch_capture",
              "xtg_batch_replay", "xtg_batch_get_info", "xtg_batch_destroy", "xtg_fill_random"):
        getattr(L, n).restype = C.c_int


class Batch:
    def __init__(self, template, reduce: str | None = None, **reduce_kw):
        self.L = lib()
        _sigs(self.L)
        ex, keep = lower(as_expr(template))
        self._keep = [ex, keep]
        rd = None
        if reduce is not None:
            reduce_kw.setdefault("axes", [-1])
            rd = make_desc(reduce, **reduce_kw)
            self._keep.append(rd)
        h = C.c_void_p()
        check(self.L.xtg_batch_create(C.byref(ex), C.byref(rd) if rd is not None else None, C.byref(h)))
        self.h = h.value

    def add(self, e, out) -> None:
        ex, keep = lower(as_expr(e))
        arr = (Array * max(ex.n_leaves, 1))()
        for i in range(ex.n_leaves):
            arr[i] = ex.leaves[i]
        o = out.xtg_array()
        check(self.L.xtg_batch_add(self.h, arr, ex.n_leaves, C.byref(o)))
        self._keep.append((keep, out))

    def build(self, autotune: bool = True, stream=None) -> "Batch":
        check(self.L.xtg_batch_build(self.h, 1 if autotune else 0, _sh(stream)))
        return self

    def run(self, stream=None) -> None:
        check(self.L.xtg_batch_run(self.h, _sh(stream)))

    def capture(self, stream: Stream) -> None:
        check(self.L.xtg_batch_capture(self.h, _sh(stream)))

    def replay(self, stream: Stream) -> None:
        check(self.L.xtg_batch_replay(self.h, _sh(stream)))

    def info(self) -> dict:
        i = BatchInfo()
        check(self.L.xtg_batch_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in BatchInfo._fields_ if k != "pad"}

    def close(self) -> None:
        if self.h:
            self.L.xtg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


DIST = {"uniform": 0, "normal": 1, "signed_lognormal": 2, "integers": 3}


def fill_random(a, dist: str, p0: float, p1: float, seed: int, stream=None):
    """Seeded synthetic data written on the device (xtg_fill_random)."""
    L = lib()
    _sigs(L)
    x = a.xtg_array()
    check(L.xtg_fill_random(C.byref(x), DIST[dist], float(p0), float(p1), int(seed) & (2**64 - 1), _sh(stream)))
    return a
