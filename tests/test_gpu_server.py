"""The request server on the GPU: every result is the same alone and in a
concurrent mix.

A set of mixed requests (assignments, row/axis/full reductions, argmax;
float32 / float64 / int32; small to medium sizes) is first evaluated one at
a time through the direct entry points ("alone"), then submitted all at once
to the server, where they are admitted as slots and budget free up, grouped
into batched launches when small and alike, and overlapped on several
streams ("in the mix").  Tolerance: elementwise results, integer results and
indices bit-exact; floating-point reductions within 1e-6 * sum|x| (the
grouped launch may sum in a different order than the standalone kernel).
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.device import DeviceArray
from xtensor_gb300.server import Server

pytestmark = pytest.mark.gpu


def make_requests(seed=11, n=120):
    g = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        kind = g.integers(0, 6)
        dt = ["float32", "float32", "float64", "int32"][g.integers(0, 4)]
        r = int(g.integers(1, 300))
        c = int(g.integers(16, 1500))

        def arr(shape):
            if dt == "int32":
                return DeviceArray.from_numpy(g.integers(-1000, 1000, shape).astype(np.int32))
            return DeviceArray.from_numpy(g.standard_normal(shape).astype(dt))

        A, v, Cm = arr((r, c)), arr((c,)), arr((r, c))
        if kind == 0:  # A * v + C, row sums (the batching expression)
            reqs.append(("reduce", "sum", A * v + Cm, [1], (r,), A, v, Cm))
        elif kind == 1:  # elementwise assignment
            e = A * v + Cm if dt == "int32" else A * v + xg.exp(-(Cm * Cm))
            reqs.append(("assign", None, e, None, (r, c), A, v, Cm))
        elif kind == 2:  # full reduction
            reqs.append(("reduce", "sum" if dt == "int32" else "variance", A, None, (), A, v, Cm))
        elif kind == 3:  # reduction over the leading axis
            reqs.append(("reduce", "amax", A, [0], (c,), A, v, Cm))
        elif kind == 4:  # arg-reduction
            reqs.append(("argmax", None, A, 1, (r,), A, v, Cm))
        else:  # transpose copy
            reqs.append(("assign", None, A.transpose(), None, (c, r), A, v, Cm))
    return reqs


def alone(req):
    kind, op, e, axes, shape = req[:5]
    if kind == "assign":
        o = DeviceArray.empty(shape, xg.expr_dtype(e))
        xg.assign(o, e)
        return o.to_numpy()
    if kind == "argmax":
        return ops.argreduce("argmax", e, axes).to_numpy()
    return ops.reduce(op, e, axes).to_numpy()


def test_results_same_alone_and_in_the_mix():
    xg.init(0)
    reqs = make_requests()
    ref = [alone(q) for q in reqs]
    srv = Server(streams=6, max_inflight=32, batch_min_group=3)
    xg.set_option("server.compile_inline", 1)  # the burst batches on its first wave
    outs, ids = [], []
    # hold admissions while the first half arrives (a burst the scheduler
    # admits together), then let the rest arrive while those run
    xg.set_option("server.paused", 1)
    for k, q in enumerate(reqs):
        if k == len(reqs) // 2:
            xg.set_option("server.paused", 0)
        kind, op, e, axes, shape = q[:5]
        if kind == "assign":
            o = DeviceArray.empty(shape, xg.expr_dtype(e))
            ids.append(srv.submit_assign(o, e))
        elif kind == "argmax":
            o = DeviceArray.empty(shape, "int64")
            ids.append(srv.submit_argreduce("argmax", e, o, axis=axes))
        else:
            sh, code = ops.reduce_shape(op, e, axes=axes)
            o = DeviceArray.empty(sh, code)
            ids.append(srv.submit_reduce(op, e, o, axes=axes))
        outs.append(o)
    results = [srv.wait(i, 120000) for i in ids]
    assert all(r["status"] == 0 for r in results)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["inflight"] == 0 and st["hbm_reserved"] == 0
    assert st["batch_launches"] >= 1, st
    xg.set_option("server.compile_inline", 0)
    for q, o, r, res in zip(reqs, outs, ref, results):
        kind, op, e, axes, shape, A, v, Cm = q
        got = o.to_numpy()
        if got.dtype.kind in "iu" or kind == "assign" or op == "amax":
            np.testing.assert_array_equal(got, r, err_msg=f"{kind} {op} batched={res['batched']}")
        else:
            a = A.to_numpy().astype(np.float64)
            if op == "sum":
                x = a * v.to_numpy() + Cm.to_numpy()
                bound = 1e-6 * np.abs(x).sum(1)
            else:
                bound = 1e-6 * np.abs(r)
            assert (np.abs(got - r) <= bound).all(), (kind, op, res)
    srv.close()


def test_admission_under_a_tight_budget():
    xg.init(0)
    g = np.random.default_rng(12)
    arrays = [DeviceArray.from_numpy(g.standard_normal((256, 1024)).astype(np.float32)) for _ in range(24)]
    srv = Server(streams=4, hbm_budget=(1 << 20) * 4, max_inflight=64)
    ids, outs = [], []
    for a in arrays:
        o = DeviceArray.empty((1024,), "float32")
        ids.append(srv.submit_reduce("sum", a, o, axes=[0], workspace=1 << 20))
        outs.append(o)
    for i in ids:
        assert srv.wait(i, 60000)["status"] == 0
    st = srv.stats()
    assert st["completed"] == 24 and st["hbm_reserved"] == 0
    assert st["waves"] >= 6  # at most ~3 fit the budget at a time
    for a, o in zip(arrays, outs):
        x = a.to_numpy().astype(np.float64)
        assert (np.abs(o.to_numpy() - x.sum(0)) <= 1e-6 * np.abs(x).sum(0)).all()
    srv.close()
