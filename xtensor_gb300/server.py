"""Python binding of the request server (xtg_server_*)."""
from __future__ import annotations

import ctypes as C

from ._ffi import Array, Expr, ReduceDesc, check, lib
from .expr import as_expr, lower
from .ops import make_desc

ASSIGN, REDUCE, ARGREDUCE = 0, 1, 2


class ServerConfig(C.Structure):
    _fields_ = [("streams", C.c_int32), ("max_inflight", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("batch_max_elems", C.c_int64), ("batch_min_group", C.c_int32), ("pad", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("arg_op", C.c_int32), ("has_axis", C.c_int32), ("pad", C.c_int32),
                ("axis", C.c_int64), ("workspace_bytes", C.c_int64), ("expr", Expr), ("rd", ReduceDesc),
                ("out", Array)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("batched", C.c_int32), ("queue_ms", C.c_double), ("total_ms", C.c_double)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "rejected", "cancelled", "inflight",
                                         "pending", "waves", "batched_requests", "batch_launches", "hbm_budget",
                                         "hbm_reserved")] + [(n, C.c_double) for n in ("p50_ms", "p99_ms", "mean_ms", "dispatch_ms")]


def _sigs(L):
    P, vp = C.POINTER, C.c_void_p
    L.xtg_server_create.argtypes = [P(ServerConfig), P(vp)]
    L.xtg_server_submit.argtypes = [vp, P(Request), P(C.c_uint64)]
    L.xtg_server_wait.argtypes = [vp, C.c_uint64, C.c_int64, P(Result)]
    L.xtg_server_cancel.argtypes = [vp, C.c_uint64]
    L.xtg_server_drain.argtypes = [vp, C.c_int64]
    L.xtg_server_get_stats.argtypes = [vp, P(Stats)]
    L.xtg_server_reset_stats.argtypes = [vp]
    L.xtg_server_destroy.argtypes = [vp]
    for n in ("xtg_server_create", "xtg_server_submit", "xtg_server_wait", "xtg_server_cancel", "xtg_server_drain",
              "xtg_server_get_stats", "xtg_server_reset_stats", "xtg_server_destroy"):
        getattr(L, n).restype = C.c_int


class Server:
    def __init__(self, streams=8, max_inflight=256, hbm_budget=0, batch_max_elems=1 << 20, batch_min_group=4):
        self.L = lib()
        _sigs(self.L)
        cfg = ServerConfig(streams, max_inflight, hbm_budget, batch_max_elems, batch_min_group, 0)
        h = C.c_void_p()
        check(self.L.xtg_server_create(C.byref(cfg), C.byref(h)))
        self.h = h.value
        self._keep = {}

    def _submit(self, req: Request, keep) -> int:
        rid = C.c_uint64()
        check(self.L.xtg_server_submit(self.h, C.byref(req), C.byref(rid)))
        self._keep[rid.value] = keep
        return rid.value

    def request(self, kind, e, out, op=None, axes=None, arg_axis=None, workspace=0, **kw) -> Request:
        ex, keep = lower(as_expr(e))
        r = Request()
        r.kind = kind
        r.expr = ex
        r.out = out.xtg_array()
        r.workspace_bytes = workspace
        if kind == REDUCE:
            r.rd = make_desc(op, axes=axes, **kw)
        elif kind == ARGREDUCE:
            r.arg_op = 0 if op == "argmax" else 1
            r.has_axis = 0 if arg_axis is None else 1
            r.axis = 0 if arg_axis is None else arg_axis
        return r, (keep, out)

    def submit_assign(self, out, e, workspace=0) -> int:
        r, keep = self.request(ASSIGN, e, out, workspace=workspace)
        return self._submit(r, keep)

    def submit_reduce(self, op, e, out, axes=None, workspace=0, **kw) -> int:
        r, keep = self.request(REDUCE, e, out, op=op, axes=axes, workspace=workspace, **kw)
        return self._submit(r, keep)

    def submit_argreduce(self, op, e, out, axis=None) -> int:
        r, keep = self.request(ARGREDUCE, e, out, op=op, arg_axis=axis)
        return self._submit(r, keep)

    def wait(self, rid: int, timeout_ms: int = -1) -> dict:
        res = Result()
        st = self.L.xtg_server_wait(self.h, rid, timeout_ms, C.byref(res))
        if st != 10:  # a timeout leaves the request alive
            self._keep.pop(rid, None)
        check(st)
        return {"status": res.status, "batched": bool(res.batched), "queue_ms": res.queue_ms, "total_ms": res.total_ms}

    def cancel(self, rid: int) -> None:
        check(self.L.xtg_server_cancel(self.h, rid))

    def drain(self, timeout_ms: int = -1) -> None:
        check(self.L.xtg_server_drain(self.h, timeout_ms))

    def stats(self) -> dict:
        s = Stats()
        check(self.L.xtg_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def reset_stats(self) -> None:
        check(self.L.xtg_server_reset_stats(self.h))

    def close(self) -> None:
        if self.h:
            self.L.xtg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
