"""K13 (k_reduce_stream) against K3 (k_reduce_row with a 256-thread group).

A full reduction of one contiguous array in 16-byte vectors with a
double-float accumulator streams through shared memory: a producer warp
copies stages of 1024 vectors with cp.async.bulk, eight consumer warps fold
them.  Each consumer thread folds the vectors and in the order a K3 thread
folds them, and the consumers combine with K3's tree, so the two kernels'
results must be equal bit for bit.  Sizes cover one item per block and
several, a last stage of a few vectors, and a work item shorter than a
stage; the error word must stay clear.
"""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import check, last_kernels
from xtensor_gb300.device import DeviceArray

pytestmark = pytest.mark.gpu

OPS = ["sum", "mean", "variance", "stddev", "norm_l1", "norm_l2", "norm_sq"]
# elements: 2^22, 2^26 + 4 * 1000 (a short last stage), 2^24 * 3 (items of
# unequal count per block), 8 * 2048 + 8.  With the default partition only
# the two large sizes stream (work items of >= 2048 vectors); with
# reduce.cta_chunk = 64 every size does, with work items shorter than a stage.
SIZES = [1 << 22, (1 << 26) + 4000, 3 << 24, 16392]


def _run(op, dx, stream_on):
    xg.set_option("reduce.stream", 1 if stream_on else 0)
    try:
        r = ops.reduce(op, dx).to_numpy()
        ks = last_kernels()
    finally:
        xg.set_option("reduce.stream", -1)
    return r, ks


@pytest.mark.parametrize("cta_chunk", [None, 64])
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dt", ["float32", "bfloat16"])
def test_stream_equals_row_kernel(n, dt, cta_chunk):
    xg.init(0)
    g = np.random.default_rng(131)
    x = (g.lognormal(0.0, 2.0, n) * np.where(g.random(n) < 0.5, -1.0, 1.0)).astype(np.float32)
    if dt == "bfloat16":
        from util import f32_to_bf16_bits
        x = f32_to_bf16_bits(x)
    dx = DeviceArray.from_numpy(x, dt)
    if cta_chunk is not None:
        xg.set_option("reduce.cta_chunk", cta_chunk)
    try:
        for op in OPS:
            a, ka = _run(op, dx, True)
            b, kb = _run(op, dx, False)
            if cta_chunk is not None or n >= (1 << 25):
                assert ka[0].startswith("k_reduce_stream<"), ka
                assert kb[0].startswith("k_reduce_row<") and ", 256, " in kb[0], kb
            assert a.tobytes() == b.tobytes(), (op, n, dt, a, b)
    finally:
        xg.set_option("reduce.cta_chunk", -1)
    check(xg.lib().xtg_check_device_errors())


@pytest.mark.parametrize("stages", [2, 3, 5, 6])
def test_ring_depths(stages):
    # 2-6 stages of 16 KiB (3 stages: exactly 48 KiB of dynamic shared
    # memory beside the kernel's static barriers); results as K3's
    xg.init(0)
    g = np.random.default_rng(132)
    x = g.standard_normal((1 << 25) + 4000).astype(np.float32)
    dx = DeviceArray.from_numpy(x)
    xg.set_option("reduce.stream_stages", stages)
    try:
        for op in ("sum", "variance", "norm_l2"):
            a, ka = _run(op, dx, True)
            b, kb = _run(op, dx, False)
            assert ka[0].startswith("k_reduce_stream<") and ka[0].split(",")[-1].strip() == f"{stages}>", ka
            assert a.tobytes() == b.tobytes(), (op, stages)
    finally:
        xg.set_option("reduce.stream_stages", -1)
    check(xg.lib().xtg_check_device_errors())
