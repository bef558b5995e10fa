"""xtensor_gb300 — GB300 evaluator for xtensor's assign + reduce hot path.

The product is ``lib/libxtg.so`` (C ABI declared in ``include/xtg.h``) and the
header-only C++ ``xt::`` surface under ``include/xtensor_gb300``.  This module
is the Python binding of the same C ABI (ctypes), used by the tests, the bench
and Python callers.  It mirrors xtensor's vocabulary: arrays with shapes and
strides in elements, lazy expressions (``xfunction``), reducers
(``sum/mean/variance/amax/norm_l2``...), ``argmax``.

There is no CPU fallback: every evaluation goes through libxtg on the GPU and
fails loudly when the library or the device is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from ._ffi import (  # noqa: F401
    ARG_MAX,
    ARG_MIN,
    DTYPES,
    Array,
    Expr,
    JitStats,
    Node,
    ReduceDesc,
    Value,
    XtgError,
    check,
    jit_stats,
    lib,
    np_dtype,
    dtype_code,
    set_option,
)
from .expr import *  # noqa: F401,F403
from .device import DeviceArray, Stream, device_sync, init  # noqa: F401
from .ops import assign, reduce, argreduce, reduce_shape, broadcast_shape, expr_dtype  # noqa: F401
from .ops import accumulate, cumsum, cumprod, nancumsum, nancumprod  # noqa: F401
from .ops import index_view, index_assign, filter_count, filter, filter_assign, masked_assign  # noqa: F401,A004
from .ops import load_npy, dump_npy, npy_header, npy_format_header  # noqa: F401
from .ops import blockwise, blockwise_shape  # noqa: F401

__all__ = [n for n in dir() if not n.startswith("_")]
