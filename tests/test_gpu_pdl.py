"""Programmatic dependent launch (option launch.pdl, on by default).

Every library kernel is launched so that the driver may set it up while the
kernel before it in the stream drains; each kernel waits on entry
(griddepcontrol.wait) until its predecessors have finished and their writes
are visible.  So the results of dependent work must be those of plain stream
order: a chain in which every step reads what the step before it wrote —
assignments, transposes, reductions of every kernel family, fused
assign + reduce, one-pass moments, chunked assignment — must give the same
bytes with the option on and off.
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.chunked import ChunkedArray
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu


def chain(seed):
    g = np.random.default_rng(seed)
    x = DeviceArray.from_numpy(g.standard_normal((384, 1024)).astype(np.float32))
    y = DeviceArray.empty((384, 1024), "float32")
    z = DeviceArray.empty((384, 1024), "float32")
    e = DeviceArray.empty((384, 1024), "float32")
    t = DeviceArray.empty((1024, 384), "float32")
    big = DeviceArray.from_numpy(g.standard_normal(1 << 24).astype(np.float32))
    c = ChunkedArray((384, 1024), (100, 96), "float32")
    outs = []
    for k in range(12):
        xg.assign(y, x * 1.0001 + 0.5)                           # K1 reads the previous step's x
        r_row = ops.reduce("sum", y, [1])                        # K3 reads y
        xg.assign(t, y.transpose((1, 0)))                        # K2 reads y
        r_col = ops.reduce("amax", t, [0])                       # K4 reads t
        arg = ops.argmax(t, 1)                                   # arg-reduction reads t
        xg.assign(z, (y - xg.rmean(y)) / xg.sqrt(xg.rvar(y) + 1e-5))  # K7 rows read y
        r_f = ops.assign_reduce(e, z * 2.0, "sum", axes=[1])     # fused: reads z, writes e
        xg.assign(big, big * 0.999 + 0.001)
        m = ops.reduce_moments(big)                              # K13, one pass
        c.assign(e * 0.5)                                        # K12 reads e
        c.to_device(x)                                           # K12 reads the chunks into x
        outs += [r_row.to_numpy(), r_col.to_numpy(), arg.to_numpy(), r_f.to_numpy()]
        outs += [v.to_numpy() for v in m.values()]
    return outs + [x.to_numpy(), y.to_numpy(), z.to_numpy(), t.to_numpy(), big.to_numpy()]


def test_dependent_chain_same_with_and_without_pdl():
    xg.init(0)
    xg.set_option("launch.pdl", 0)
    try:
        off = chain(91)
    finally:
        xg.set_option("launch.pdl", -1)
    on = chain(91)
    assert len(on) == len(off)
    for i, (a, b) in enumerate(zip(on, off)):
        assert a.dtype == b.dtype and a.shape == b.shape, i
        assert a.tobytes() == b.tobytes(), i
