"""The compiled CPU port of the reference's loops (oracle/xt_baseline.c) pinned
to the oracle on small seeded inputs.

bench.py times the port as the CPU baseline and checks the GPU results of the
benchmark steps against the port's outputs, so the port has to compute what
the reference computes.  Here every port routine the benchmarks use is
compared with the oracle's restatement of the reference
(oracle/xt_oracle.c) on the same inputs:

  * transpose, amax over {0, 2}, argmax over axis 1: bit-exact;
  * the row normalisation (x - mean) / sqrt(var + 1e-5): bit-exact (both
    follow the reference: sequential row sum in the value type, mean and
    variance in double, the tree in double, one cast);
  * C0's E = A * b + exp(-A * A) and its row sums: bit-exact (the same
    libm expf, the same sequential float fold);
  * one C3 instance, sum(A * v + C, {1}): bit-exact;
  * full float32 / int32 -> int64 sums: bit-exact (sequential folds);
  * the precision workload's sum / mean / variance / norm_l2 of float32
    and bfloat16 arrays: bit-exact;
  * cumsum along each axis and flattened: bit-exact;
  * chunked arrays (assignment chunk by chunk, reading, sum over the last
    axis): bit-exact, the padding of edge chunks untouched.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300.device import HostArray
from oracle import oracle as O

P = C.c_void_p
I64 = C.c_int64


def port():
    O.lib()
    L = C.CDLL(str(O.SO))
    for t in ("f32", "f64"):
        getattr(L, f"bl_transpose_201_{t}").argtypes = [P, P, I64, I64, I64]
        getattr(L, f"bl_amax_02_{t}").argtypes = [P, P, I64, I64, I64]
        getattr(L, f"bl_normalize_{t}").argtypes = [P, P, I64, I64, C.c_double]
        getattr(L, f"bl_argmax_1_{t}").argtypes = [P, P, I64, I64, I64, P]
    L.bl_c0_assign.argtypes = [P, P, P, I64, I64]
    L.bl_c0_sum.argtypes = [P, P, I64, I64]
    L.bl_c3_rowsum_f32.argtypes = [P, P, P, P, I64, I64]
    L.bl_sum_f32.argtypes = [P, I64]
    L.bl_sum_f32.restype = C.c_float
    L.bl_sum_i32_i64.argtypes = [P, I64]
    L.bl_sum_i32_i64.restype = C.c_int64
    for t in ("f32", "f64", "i32"):
        getattr(L, f"bl_cumsum_{t}").argtypes = [P, P, I64, I64, I64, C.c_int]
    for t in ("f32", "bf16"):
        for op in ("sum", "mean", "variance", "norm_l2"):
            f = getattr(L, f"bl_stat_{op}_{t}")
            f.argtypes = [P, I64]
            f.restype = C.c_float if op == "sum" else C.c_double
    return L


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


SHAPES = [(6, 10, 33), (3, 17, 64), (1, 1, 5)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_port_c1_step_equals_oracle(shape, dt):
    L = port()
    t = "f32" if dt == "float32" else "f64"
    g = np.random.default_rng(101)
    x = g.standard_normal(shape).astype(dt)
    x[0, 0, 0] = -0.0
    d0, d1, d2 = shape
    h = HostArray(x)

    tr = np.empty((d2, d0, d1), dt)
    getattr(L, f"bl_transpose_201_{t}")(ptr(x), ptr(tr), d0, d1, d2)
    ref_t = O.assign(HostArray(x.transpose(2, 0, 1)))
    np.testing.assert_array_equal(tr.view(np.uint8), ref_t.view(np.uint8))

    y = np.empty(shape, dt)
    getattr(L, f"bl_normalize_{t}")(ptr(x), ptr(y), d0 * d1, d2, 1e-5)
    ref_y = O.assign((h - xg.rmean(h)) / xg.sqrt(xg.rvar(h) + 1e-5), dtype=dt)
    np.testing.assert_array_equal(y.view(np.uint8), ref_y.view(np.uint8))

    am = np.empty((d1,), dt)
    getattr(L, f"bl_amax_02_{t}")(ptr(x), ptr(am), d0, d1, d2)
    ref_am = O.reduce("amax", h, [0, 2])
    np.testing.assert_array_equal(am.view(np.uint8), ref_am.view(np.uint8))

    ai = np.empty((d0, d2), np.int32)
    tmp = np.empty((d0, d2, d1), dt)
    getattr(L, f"bl_argmax_1_{t}")(ptr(x), ptr(ai), d0, d1, d2, ptr(tmp))
    np.testing.assert_array_equal(ai, O.argreduce("argmax", h, 1))


@pytest.mark.parametrize("n,m", [(37, 45), (8, 2048), (1, 1)])
def test_port_c0_equals_oracle(n, m):
    L = port()
    g = np.random.default_rng(0)
    A = g.uniform(-1, 1, (n, m)).astype(np.float32)
    b = g.standard_normal(m).astype(np.float32)
    E = np.empty((n, m), np.float32)
    L.bl_c0_assign(ptr(A), ptr(b), ptr(E), n, m)
    hA, hb = HostArray(A), HostArray(b)
    ref_E = O.assign(hA * hb + xg.exp(-hA * hA))
    np.testing.assert_array_equal(E, ref_E)
    r = np.empty((n,), np.float32)
    L.bl_c0_sum(ptr(E), ptr(r), n, m)
    np.testing.assert_array_equal(r, O.reduce("sum", HostArray(E), [1]))


@pytest.mark.parametrize("n,m", [(1, 16), (37, 45), (5, 2048)])
def test_port_c3_instance_equals_oracle(n, m):
    L = port()
    g = np.random.default_rng(3)
    A = g.uniform(-1, 1, (n, m)).astype(np.float32)
    v = g.standard_normal(m).astype(np.float32)
    Cm = g.uniform(-1, 1, (n, m)).astype(np.float32)
    r = np.empty((n,), np.float32)
    L.bl_c3_rowsum_f32(ptr(A), ptr(v), ptr(Cm), ptr(r), n, m)
    want = O.reduce("sum", HostArray(A) * HostArray(v) + HostArray(Cm), [1])
    np.testing.assert_array_equal(r, want)


def test_port_full_sums_equal_oracle():
    L = port()
    g = np.random.default_rng(2)
    x = (g.lognormal(0, 2, 10007) * g.choice([-1, 1], 10007)).astype(np.float32)
    got = np.float32(L.bl_sum_f32(ptr(x), x.size))
    assert got.view(np.uint32) == O.reduce("sum", HostArray(x)).astype(np.float32).view(np.uint32)
    i = g.integers(-(2**20), 2**20 + 1, 10007).astype(np.int32)
    assert L.bl_sum_i32_i64(ptr(i), i.size) == int(O.reduce("sum", HostArray(i), acc_dtype="int64"))


@pytest.mark.parametrize("dt", ["float32", "float64", "int32"])
@pytest.mark.parametrize("axis", [0, 1, 2, -1])
def test_port_cumsum_equals_oracle(dt, axis):
    L = port()
    t = {"float32": "f32", "float64": "f64", "int32": "i32"}[dt]
    g = np.random.default_rng(5)
    shape = (4, 9, 13)
    x = g.standard_normal(shape).astype(dt) if dt != "int32" else g.integers(-1000, 1001, shape).astype(dt)
    r = np.empty(shape, dt)
    getattr(L, f"bl_cumsum_{t}")(ptr(x), ptr(r), *shape, axis)
    ref = O.accumulate("cumsum", HostArray(x), None if axis < 0 else axis)
    np.testing.assert_array_equal(r.reshape(ref.shape), ref)


@pytest.mark.parametrize("dt", ["float32", "bfloat16"])
@pytest.mark.parametrize("n", [1, 7, 10007])
def test_port_precision_stats_equal_oracle(dt, n):
    from util import f32_to_bf16_bits
    L = port()
    g = np.random.default_rng(2)
    x = (g.lognormal(0, 2, n) * g.choice([-1, 1], n)).astype(np.float32)
    arr, t = (x, "f32") if dt == "float32" else (f32_to_bf16_bits(x), "bf16")
    h = HostArray(arr, dt)
    for op in ("sum", "mean", "variance", "norm_l2"):
        got = getattr(L, f"bl_stat_{op}_{t}")(ptr(arr), n)
        ref = O.reduce(op, h)
        want = ref.astype(np.float32 if op == "sum" else np.float64)
        got = np.asarray(got, dtype=want.dtype)
        assert got.tobytes() == want.tobytes(), (op, dt, n, got, want)


@pytest.mark.parametrize("shape,cs", [((9, 10, 11), (4, 3, 5)), ((8, 6, 16), (4, 3, 8)), ((5, 7, 3), (8, 8, 8))])
def test_port_chunked_equals_oracle(shape, cs):
    from oracle import chunked as OC
    O.lib()
    L = C.CDLL(str(O.SO))
    PP = C.POINTER(C.c_void_p)
    L.bl_chunked_axpb_f32.argtypes = [P, PP, P, P, C.c_float, C.c_float]
    L.bl_chunked_read_f32.argtypes = [PP, P, P, P]
    L.bl_chunked_sum2_f32.argtypes = [PP, P, P, P]
    g = np.random.default_rng(71)
    x = g.standard_normal(shape).astype(np.float32)
    n = int(np.prod(OC.grid_shape(shape, cs)))
    chunks = [np.full(cs, -5.0, np.float32) for _ in range(n)]
    tab = (C.c_void_p * n)(*[c.ctypes.data for c in chunks])
    d = np.array(shape, np.int64)
    c = np.array(cs, np.int64)
    L.bl_chunked_axpb_f32(ptr(x), tab, ptr(d), ptr(c), 2.0, 1.0)
    vals = O.assign(HostArray(x) * np.float32(2.0) + np.float32(1.0))
    want = OC.assign_chunks([np.full(cs, -5.0, np.float32) for _ in range(n)], vals, cs)
    for u, v in zip(chunks, want):
        assert u.tobytes() == v.tobytes()  # the padding of edge chunks untouched
    dense = np.empty(shape, np.float32)
    L.bl_chunked_read_f32(tab, ptr(dense), ptr(d), ptr(c))
    np.testing.assert_array_equal(dense, vals)
    s2 = np.empty(shape[:2], np.float32)
    L.bl_chunked_sum2_f32(tab, ptr(s2), ptr(d), ptr(c))
    np.testing.assert_array_equal(s2, O.reduce("sum", HostArray(vals), [2]))
