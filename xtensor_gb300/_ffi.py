"""ctypes mirror of include/xtg.h."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

MAX_RANK = 8
MAX_LEAVES = 8
MAX_NODES = 48

# xtg_dtype codes
DTYPES = {
    "bool": 0, "int8": 1, "uint8": 2, "int16": 3, "uint16": 4, "int32": 5, "uint32": 6,
    "int64": 7, "uint64": 8, "bfloat16": 9, "float32": 10, "float64": 11,
}
_NP = {
    0: np.bool_, 1: np.int8, 2: np.uint8, 3: np.int16, 4: np.uint16, 5: np.int32, 6: np.uint32,
    7: np.int64, 8: np.uint64, 9: np.uint16, 10: np.float32, 11: np.float64,
}
ITEMSIZE = {k: np.dtype(v).itemsize for k, v in _NP.items()}

# opcodes
OP = dict(
    LEAF=0, SCALAR=1,
    NEG=10, POS=11, EXP=12, LOG=13, SQRT=14, ABS=15, SQUARE=16, SIN=17, COS=18, TANH=19,
    LOGICAL_NOT=20, BIT_NOT=21, CAST=22,
    ADD=40, SUB=41, MUL=42, DIV=43, MOD=44, MAXIMUM=45, MINIMUM=46, LT=47, LE=48, GT=49, GE=50,
    EQ=51, NE=52, LOGICAL_AND=53, LOGICAL_OR=54, BIT_AND=55, BIT_OR=56, BIT_XOR=57, POW=58,
    WHERE=70,
    RSUM=80, RMEAN=81, RVAR=82, RSTD=83, RMAX=84, RMIN=85,
)
RED = dict(sum=0, prod=1, amax=2, amin=3, mean=4, variance=5, stddev=6,
           norm_l0=7, norm_l1=8, norm_sq=9, norm_l2=10, norm_linf=11,
           norm_lp_to_p=12, norm_lp=13)  # the last two: blockwise only
ARG_MAX, ARG_MIN = 0, 1
PREC_COMPENSATED, PREC_PLAIN = 0, 1

STATUS = {
    0: "ok", 1: "invalid argument", 2: "broadcast error", 3: "invalid reduction axes",
    4: "axis out of range", 5: "shape mismatch", 6: "CUDA error", 7: "kernel compilation failed",
    8: "out of device memory", 9: "unsupported", 10: "timeout", 11: "rejected", 12: "cancelled",
    13: "not found",
}


def np_dtype(code: int):
    return _NP[code]


def dtype_code(d) -> int:
    if isinstance(d, int):
        return d
    if isinstance(d, str):
        return DTYPES[d]
    d = np.dtype(d)
    for k, v in _NP.items():
        if k != 9 and np.dtype(v) == d:
            return k
    raise TypeError(f"unsupported dtype {d}")


class Value(C.Union):
    _fields_ = [("f", C.c_double), ("i", C.c_int64), ("u", C.c_uint64)]


class Node(C.Structure):
    _fields_ = [("op", C.c_int32), ("dtype", C.c_int32), ("arg", C.c_int32), ("aux", C.c_int32), ("imm", Value)]


class Array(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int32), ("rank", C.c_int32),
                ("shape", C.c_int64 * MAX_RANK), ("strides", C.c_int64 * MAX_RANK)]


class Expr(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_leaves", C.c_int32),
                ("nodes", Node * MAX_NODES), ("leaves", Array * MAX_LEAVES)]


class ReduceDesc(C.Structure):
    _fields_ = [("op", C.c_int32), ("n_axes", C.c_int32), ("axes", C.c_int64 * MAX_RANK),
                ("keep_dims", C.c_int32), ("has_initial", C.c_int32), ("initial", Value),
                ("acc_dtype", C.c_int32), ("precision", C.c_int32), ("ddof", C.c_int64)]


class NpyHeader(C.Structure):
    _fields_ = [("descr", C.c_char * 16), ("dtype", C.c_int32), ("fortran_order", C.c_int32),
                ("version", C.c_int32), ("rank", C.c_int32), ("shape", C.c_int64 * MAX_RANK),
                ("data_offset", C.c_int64), ("data_bytes", C.c_int64)]


LAYOUTS = {"dynamic": 0, "row_major": 1, "column_major": 2}


class JitStats(C.Structure):
    _fields_ = [("compiles", C.c_int64), ("disk_hits", C.c_int64), ("memory_hits", C.c_int64),
                ("compile_seconds", C.c_double), ("launches", C.c_int64)]


class XtgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "lib" / "libxtg.so"


def lib() -> C.CDLL:
    """Load libxtg.so (built in-tree by xtensor_gb300/build.py)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m xtensor_gb300.build` first")
        L = C.CDLL(str(LIB_PATH))
        vp, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
        st = C.c_int
        sig = {
            "xtg_version": (C.c_char_p, []),
            "xtg_status_string": (C.c_char_p, [st]),
            "xtg_last_error": (C.c_char_p, []),
            "xtg_init": (st, [C.c_int]),
            "xtg_device_count": (st, [C.POINTER(C.c_int)]),
            "xtg_device_info": (st, [C.POINTER(C.c_int), C.POINTER(i64), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
            "xtg_mem_info": (st, [C.POINTER(i64), C.POINTER(i64)]),
            "xtg_malloc": (st, [C.POINTER(vp), sz, vp]),
            "xtg_free": (st, [vp, vp]),
            "xtg_host_alloc": (st, [C.POINTER(vp), sz]),
            "xtg_host_free": (st, [vp]),
            "xtg_memcpy": (st, [vp, vp, sz, C.c_int, vp]),
            "xtg_memset": (st, [vp, C.c_int, sz, vp]),
            "xtg_stream_create": (st, [C.POINTER(vp)]),
            "xtg_stream_destroy": (st, [vp]),
            "xtg_stream_sync": (st, [vp]),
            "xtg_device_sync": (st, []),
            "xtg_dtype_size": (sz, [i32]),
            "xtg_broadcast_shape": (st, [C.POINTER(Expr), C.POINTER(i32), C.POINTER(i64)]),
            "xtg_expr_dtype": (st, [C.POINTER(Expr), C.POINTER(i32)]),
            "xtg_reduce_shape": (st, [C.POINTER(Expr), C.POINTER(ReduceDesc), C.POINTER(i32), C.POINTER(i64), C.POINTER(i32)]),
            "xtg_reduce_acc_dtype": (st, [C.POINTER(Expr), C.POINTER(ReduceDesc), C.POINTER(i32)]),
            "xtg_assign": (st, [C.POINTER(Expr), C.POINTER(Array), vp]),
            "xtg_reduce": (st, [C.POINTER(Expr), C.POINTER(ReduceDesc), C.POINTER(Array), vp]),
            "xtg_argreduce": (st, [C.POINTER(Expr), i32, i32, i64, C.POINTER(Array), vp]),
            "xtg_assign_reduce": (st, [C.POINTER(Expr), C.POINTER(Array), C.POINTER(ReduceDesc), C.POINTER(Array), vp]),
            "xtg_reduce_moments": (st, [C.POINTER(Expr), C.POINTER(ReduceDesc), C.POINTER(Array), C.POINTER(Array),
                                        C.POINTER(Array), C.POINTER(Array), vp]),
            "xtg_accumulate_shape": (st, [C.POINTER(Expr), i32, i32, i64, i32, C.POINTER(i32), C.POINTER(i64),
                                          C.POINTER(i32)]),
            "xtg_accumulate": (st, [C.POINTER(Expr), i32, i32, i64, i32, C.POINTER(Array), vp]),
            "xtg_gather": (st, [C.POINTER(Expr), vp, i64, C.POINTER(Array), vp]),
            "xtg_scatter": (st, [C.POINTER(Expr), vp, i64, i32, C.POINTER(Array), vp]),
            "xtg_filter_count": (st, [C.POINTER(Expr), C.POINTER(i64), vp]),
            "xtg_filter": (st, [C.POINTER(Expr), C.POINTER(Expr), C.POINTER(Array), vp]),
            "xtg_filter_assign": (st, [C.POINTER(Expr), C.POINTER(Expr), i32, C.POINTER(Array), vp]),
            "xtg_masked_assign": (st, [C.POINTER(Expr), C.POINTER(Expr), i32, C.POINTER(Array), vp]),
            "xtg_npy_info": (st, [C.c_char_p, C.POINTER(NpyHeader)]),
            "xtg_npy_info_buffer": (st, [vp, sz, C.POINTER(NpyHeader)]),
            "xtg_npy_format_header": (st, [i32, i32, i32, C.POINTER(i64), vp, sz, C.POINTER(sz)]),
            "xtg_npy_load": (st, [C.c_char_p, C.POINTER(Array), i32, vp]),
            "xtg_npy_load_buffer": (st, [vp, sz, C.POINTER(Array), i32, vp]),
            "xtg_npy_save": (st, [C.c_char_p, C.POINTER(Array), vp]),
            "xtg_npy_save_buffer": (st, [C.POINTER(Array), vp, sz, C.POINTER(sz), vp]),
            "xtg_blockwise_reduce": (st, [C.POINTER(Array), C.POINTER(i64), C.POINTER(ReduceDesc), C.c_double,
                                          C.POINTER(Array), vp]),
            "xtg_blockwise_shape": (st, [C.POINTER(Array), C.POINTER(ReduceDesc), C.POINTER(i32), C.POINTER(i64),
                                         C.POINTER(i32)]),
            "xtg_get_jit_stats": (st, [C.POINTER(JitStats)]),
            "xtg_set_option": (st, [C.c_char_p, i64]),
            "xtg_get_option": (st, [C.c_char_p, C.POINTER(i64)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _extend_signatures(L)
        _LIB = L
    return _LIB


def _extend_signatures(L) -> None:
    """Signatures of optional entry points (present in later builds)."""
    vp, i32, i64, sz, st = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t, C.c_int
    extra = {
        "xtg_event_create": (st, [C.POINTER(vp)]),
        "xtg_event_destroy": (st, [vp]),
        "xtg_event_record": (st, [vp, vp]),
        "xtg_event_elapsed_ms": (st, [vp, vp, C.POINTER(C.c_float)]),
        "xtg_event_sync": (st, [vp]),
        "xtg_stream_wait_event": (st, [vp, vp]),
        "xtg_last_kernels": (C.c_char_p, []),
        "xtg_sum_f32_noalloc": (st, [vp, i64, vp, vp]),
    }
    for name, (res, args) in extra.items():
        f = getattr(L, name, None)
        if f is not None:
            f.restype = res
            f.argtypes = args


def check(status: int) -> None:
    if status != 0:
        msg = lib().xtg_last_error().decode(errors="replace")
        raise XtgError(status, msg)


def set_option(key: str, value: int) -> None:
    check(lib().xtg_set_option(key.encode(), int(value)))


def last_kernels() -> list[str]:
    """Kernels launched by the last evaluation call on this thread."""
    s = lib().xtg_last_kernels().decode()
    return [k for k in s.split(";") if k]


def jit_stats() -> dict:
    s = JitStats()
    check(lib().xtg_get_jit_stats(C.byref(s)))
    return {k: getattr(s, k) for k, _ in JitStats._fields_}
