"""Helpers shared by the tests: seeded inputs, ulp distances, bf16."""
from __future__ import annotations

import numpy as np


def rng(seed=0):
    return np.random.default_rng(seed)


def f32_to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even float32 -> bfloat16 bit patterns (uint16)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return r


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place (float32 / float64), NaN==NaN -> 0."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype == np.float32:
        ia = a.view(np.int32).astype(np.int64)
        ib = b.view(np.int32).astype(np.int64)
        ia = np.where(ia < 0, np.int64(-(2**31)) - ia, ia)
        ib = np.where(ib < 0, np.int64(-(2**31)) - ib, ib)
    else:
        ia = a.view(np.int64).astype(object)
        ib = b.view(np.int64).astype(object)
        ia = np.where(ia < 0, -(2**63) - ia, ia)
        ib = np.where(ib < 0, -(2**63) - ib, ib)
    d = np.abs(ia - ib)
    both_nan = np.isnan(a) & np.isnan(b)
    return np.where(both_nan, 0, d).astype(np.float64)


def assert_ulp(got, ref, max_ulp, what=""):
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if got.size == 0:
        return
    d = ulp_diff(got, ref)
    worst = float(d.max())
    assert worst <= max_ulp, f"{what}: max ulp distance {worst} > {max_ulp}"


def assert_close_rel(got, ref, rel, scale=None, what=""):
    """|got - ref| <= rel * scale (scale defaults to |ref|, elementwise)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    sc = np.abs(ref) if scale is None else np.asarray(scale, dtype=np.float64)
    err = np.abs(got - ref)
    ok = (err <= rel * sc) | (np.isnan(got) & np.isnan(ref)) | (got == ref)
    assert ok.all(), f"{what}: max err {err.max()} vs allowed {rel} * scale (worst idx {np.argmax(err - rel * sc)})"
