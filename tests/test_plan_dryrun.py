"""Planning and kernel compilation without a GPU.

In dry-run mode libxtg plans every call against a GB300-shaped device,
compiles the chosen kernel instantiations with NVRTC for sm_103a and skips
the launch.  These tests check which kernel family each workload of the
benchmark configurations lowers to, and that every one of them compiles."""
from __future__ import annotations

import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import last_kernels
from xtensor_gb300.device import DeviceArray


@pytest.fixture(autouse=True)
def dry():
    xg.set_option("jit.dry_run", 1)
    yield
    xg.set_option("jit.dry_run", -1)


_next = [0x100000000]


def fake(shape, dtype):
    p = _next[0]
    _next[0] += 1 << 36
    return DeviceArray(shape, dtype, p)


def fam(names):
    return [n.split("<", 1)[0] for n in names]


def test_c0_plain_small():
    A, b = fake((2048, 2048), "float32"), fake((2048,), "float32")
    E = fake((2048, 2048), "float32")
    xg.assign(E, A * b + xg.exp(-A * A))
    ks = last_kernels()
    assert fam(ks) == ["k_assign"]
    assert ", 4, 2, " in ks[0]  # 16-byte vectors over a 2-D (rows x 2048) space
    r = fake((2048,), "float32")
    ops.reduce("sum", A * b + xg.exp(-A * A), [1], out=r)  # E not materialised
    assert fam(last_kernels()) == ["k_reduce_row"]
    assert "AccSumC" in last_kernels()[0]


@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_c1_strided_axis(dt):
    x = fake((256, 512, 1024), dt)
    t = fake((1024, 256, 512), dt)
    xg.assign(t, x.transpose((2, 0, 1)))
    assert fam(last_kernels()) == ["k_transpose"]
    y = fake((256, 512, 1024), dt)
    xg.assign(y, (x - xg.rmean(x)) / xg.sqrt(xg.rvar(x) + 1e-5))
    ks = last_kernels()
    # rows of 1024 contiguous elements: the bulk-copy (TMA) variant with one
    # buffer per warp and a register bound of 5 blocks per SM (a lane holds
    # 64 registers of the row at most)
    assert fam(ks) == ["k_rowfused_tma"] and "RStat<0, 1" in ks[0] and "RStat<1, 2" in ks[0]
    assert ks[0].endswith(", 1, 5>"), ks[0]
    xg.set_option("row.tma_buffers", 2)
    xg.set_option("row.tma_min_blocks", 3)
    try:
        xg.assign(y, (x - xg.rmean(x)) / xg.sqrt(xg.rvar(x) + 1e-5))
        assert last_kernels()[0].endswith(", 2, 3>")
    finally:
        xg.set_option("row.tma_buffers", -1)
        xg.set_option("row.tma_min_blocks", -1)
    if dt == "float64":
        assert "FmaRecipSub<double" in ks[0]
    am = fake((512,), dt)
    ops.reduce("amax", x, [0, 2], out=am)
    assert fam(last_kernels())[0] == "k_reduce_row"
    ai = fake((256, 1024), "int32")
    ops.argreduce("argmax", x, 1, out=ai)
    assert fam(last_kernels())[0] == "k_reduce_col"


def test_c2_precision_full_reductions():
    n = 1 << 28
    for dt, acc in [("float32", "AccSumC"), ("bfloat16", "AccSumC")]:
        x = fake((n,), dt)
        out = fake((), "float32")
        ops.reduce("sum", x, out=out)
        ks = last_kernels()
        # 2^28 contiguous elements in 16-byte vectors: the streaming full reduction
        assert fam(ks) == ["k_reduce_stream", "k_reduce_combine"] and acc in ks[0]
        for op, a in [("mean", "AccSumC"), ("variance", "AccMom<float, 1>"), ("norm_l2", "AccNormC<2>")]:
            o = fake((), "float64")
            ops.reduce(op, x, out=o)
            assert a in last_kernels()[0], (op, last_kernels())
    xi = fake((n,), "int32")
    o = fake((), "int64")
    ops.reduce("sum", xi, acc_dtype="int64", out=o)
    assert "AccPlain<long long, 0>" in last_kernels()[0]


@pytest.mark.parametrize("dt", ["float32", "bfloat16"])
def test_c2_one_pass_moments(dt):
    # sum, mean, variance and norm_l2 of 2^28 elements: one streaming launch
    # with the four accumulators, one combine writing the four results
    x = fake((1 << 28,), dt)
    outs = {nm: fake(*ops.reduce_shape(nm, x)) for nm in ops.MOMENTS}
    ops.reduce_moments(x, outs=outs)
    ks = last_kernels()
    assert fam(ks) == ["k_reduce_stream", "k_reduce_combine"] and "AccStats" in ks[0]
    assert "StatsOut<float, double, double, double>" in ks[1]


def test_views_and_broadcast_plans():
    x = fake((64, 48), "float32")
    o = fake((32, 40), "float32")
    xg.assign(o, x[::2, 3:43] + xg.scalar(1.0, "float32"))
    assert fam(last_kernels()) == ["k_assign"]
    o2 = fake((48, 64), "float32")
    xg.assign(o2, x.transpose() * xg.scalar(2.0, "float32"))
    assert fam(last_kernels()) == ["k_transpose"]


def test_type_and_shape_errors_are_reported_before_launch():
    a = fake((3, 4), "float32")
    b = fake((5,), "float32")
    with pytest.raises(xg.XtgError) as ei:
        xg.assign(fake((3, 4), "float32"), a + b)
    assert ei.value.status == 2
    with pytest.raises(xg.XtgError) as ei:
        ops.reduce("sum", a, [1, 0], out=fake((), "float32"))
    assert ei.value.status == 3
    with pytest.raises(xg.XtgError) as ei:
        xg.assign(fake((3, 4), "float32"), a % a)
    assert ei.value.status == 1


def test_batch_plans_and_compiles():
    from xtensor_gb300.batch import Batch
    A0, v0, C0 = fake((10, 20), "float32"), fake((20,), "float32"), fake((10, 20), "float32")
    b = Batch(A0 * v0 + C0, reduce="sum")
    for r, c in [(10, 20), (1, 16), (4096, 2048), (7, 33)]:
        A, v, Cm = fake((r, c), "float32"), fake((c,), "float32"), fake((r, c), "float32")
        b.add(A * v + Cm, fake((r,), "float32"))
    b.build(autotune=False)
    info = b.info()
    assert info["instances"] == 4 and info["tiles"] >= 4
    assert info["algorithmic_bytes"] == sum(4 * (2 * r * c + c + r) for r, c in [(10, 20), (1, 16), (4096, 2048), (7, 33)])
    ba = Batch(A0 * v0 + C0)
    ba.add(A0 * v0 + C0, fake((10, 20), "float32"))
    ba.build(autotune=False)


@pytest.mark.parametrize("dt", ["float32", "float64", "int32"])
def test_accumulator_plans(dt):
    """cumsum / cumprod lower to the sequential column / row scans or the
    tile scan, and every variant compiles."""
    from xtensor_gb300 import ops
    x = fake((64, 300, 33), dt)
    for ax, fam_want in ((0, ["k_scan_col"]), (1, ["k_scan_col"]), (2, ["k_scan_rows"]),
                         (None, ["k_scan_seg_reduce", "k_scan_seg_offsets", "k_scan_seg_apply"])):
        for op in ("cumsum", "cumprod"):
            shape, odt = ops.accumulate_shape(op, x, ax)
            ops.accumulate(op, x, ax, out=fake(shape, odt))
            assert fam(last_kernels()) == fam_want, (ax, op, last_kernels())
    # a flattened transposed view is evaluated into a temporary first
    n = 64 * 300 * 33
    ops.accumulate("cumsum", x.transpose((2, 0, 1)), None, out=fake((n,), ops.accumulate_shape("cumsum", x)[1]))
    assert fam(last_kernels())[0] == "k_transpose"


def test_segmented_scan_variants():
    """The segmented scan's apply pass streams a plain contiguous operand of
    the accumulation type (4 or 8 bytes) through its cp.async ring in tiles
    of 32 x 16 (template tail: stages, elements per lane, lane folds kept by
    pass A, chains per lane); float64 keeps the lanes' folds from pass A and
    folds in two chains, with or without them; expressions and unaligned or
    strided operands take the register form (32 x 8).  Pass A's tiles match
    pass C's for streamed operands; every variant compiles."""
    from xtensor_gb300 import ops
    n = 3_000_001

    def plan(x, **opts):
        for k, v in opts.items():
            xg.set_option(k, v)
        try:
            ops.accumulate("cumsum", x, None, out=fake((x.size,), x.dtype))
            return last_kernels()
        finally:
            for k in opts:
                xg.set_option(k, -1)

    ks = plan(fake((n,), "float64"))
    assert fam(ks) == ["k_scan_seg_reduce", "k_scan_seg_offsets", "k_scan_seg_apply"]
    assert ks[0].endswith(", 2, 16, true, 2>") and ks[2].endswith(", 2, 3, 16, true, 2>"), ks
    ks = plan(fake((n,), "float64"), **{"scan.lane_totals": 0})
    assert ks[0].endswith(", 2, 16, false, 2>") and ks[2].endswith(", 2, 3, 16, false, 2>"), ks
    ks = plan(fake((n,), "float32"))
    assert ks[0].endswith(", 4, 16, false, 1>") and ks[2].endswith(", 4, 3, 16, false, 1>"), ks
    ks = plan(fake((n,), "int32"), **{"scan.seg_stages": 5})
    assert ks[2].endswith(", 4, 5, 16, false, 1>"), ks
    # the register form: no ring, 8 elements per lane in pass C (pass A
    # keeps 16 for 4-byte types: its tiles only have to cover the segments)
    ks = plan(fake((n,), "float32"), **{"scan.async": 0})
    assert ks[0].endswith(", 4, 16, false, 1>") and ks[2].endswith(", 4, 0, 8, false, 1>"), ks
    x = fake((n,), "float32")
    ops.accumulate("cumsum", x + x, None, out=fake((n,), "float32"))
    assert last_kernels()[2].endswith(", 0, 8, false, 1>"), last_kernels()
    # a strided operand: scalar loads through the warp's buffer
    y = fake((2, n), "float64")
    ops.accumulate("cumsum", y[:, ::2], 1, out=fake((2, (n + 1) // 2), "float64"))
    assert last_kernels()[-1].endswith(", 1, 0, 8, false, 1>"), last_kernels()


def test_view_plans():
    """Masked writes lower to the elementwise kernel, index views to the
    indexed kernel, filters to the accumulator (positions) + indexed kernel;
    everything compiles."""
    from xtensor_gb300 import ops
    a = fake((64, 300), "float32")
    m = fake((64, 300), "bool")
    ops.masked_assign(a, m, a * 2, "+=")
    assert fam(last_kernels()) == ["k_assign"]
    idx = fake((100, 2), "int64")
    ops.index_view(a, idx, out=fake((100,), "float32"))
    assert fam(last_kernels()) == ["k_indexed"]
    ops.index_assign(a, idx, fake((100,), "float64"), "*=")
    assert fam(last_kernels()) == ["k_indexed"]
    ops.filter(a, a > 0, out=fake((0,), "float32"))
    ks = fam(last_kernels())
    assert ks[0] == "k_filter_count" and ks[-1] == "k_filter_tile", ks
    ops.filter_assign(a, a > 0, 1.5, "=")
    assert fam(last_kernels())[-1] == "k_filter_tile"
    # a write through a transposed view of itself goes through a temporary
    sq = fake((64, 64), "float32")
    xg.assign(sq, sq.transpose((1, 0)))
    assert fam(last_kernels()) == ["k_transpose", "k_assign"]


def fake_chunked(shape, cs, dt, spaced=True):
    """A chunked array over fake device addresses: chunks at a 256-byte
    aligned distance (one slab) or scattered."""
    import math
    from xtensor_gb300._ffi import ITEMSIZE, dtype_code
    from xtensor_gb300.chunked import ChunkedArray, grid_shape
    n = math.prod(grid_shape(shape, cs))
    es = ITEMSIZE[dtype_code(dt)]
    dist = -(-math.prod(cs) * es // 256) * 256
    base = _next[0]
    _next[0] += 1 << 40
    chunks = [DeviceArray(cs, dt, base + (i * dist if spaced else i * (dist + 4096) + (i % 3) * 256)) for i in range(n)]
    return ChunkedArray(shape, cs, dt, chunks=chunks)


@pytest.mark.parametrize("shape,cs,vec,pad", [
    ((256, 512, 1024), (64, 256, 1024), 4, "false"),   # whole chunks: one class
    ((256, 512, 1024), (100, 200, 1000), 4, "false"),  # edges on every axis: 8 classes, edge of 24 divides by 4
    ((37, 70, 45), (5, 9, 7), 1, "false"),             # an odd inner extent: scalar elements
    ((3, 5, 7, 9, 11), (2, 2, 4, 3, 5), 1, "true"),    # 16 classes: padded chunks with extent tests
])
def test_chunked_assign_plan(shape, cs, vec, pad):
    # xtg_chunked_assign: one k_assign_chunks launch over the chunk classes
    x = fake(shape, "float32")
    a = fake_chunked(shape, cs, "float32")
    a.assign(x * 2.0 + 1.0)
    ks = last_kernels()
    assert fam(ks) == ["k_assign_chunks"], ks
    tail = ks[0].rsplit(">", 1)[0].split(", ")[-6:]  # OUTKIND, VEC, R, U, BIG, PAD
    assert tail[1] == str(vec) and tail[2] == str(len(shape)) and tail[5] == pad, tail


def test_chunked_full_sum_of_a_slab_is_one_streaming_reduction():
    # whole chunks in one slab: the full sum is one run of the slab (K13)
    from xtensor_gb300.chunked import chunked_reduce
    a = fake_chunked((256, 512, 1024), (64, 256, 1024), "float32")
    out = fake((), "float32")
    n0 = xg.jit_stats()["launches"]
    chunked_reduce("sum", a, out=out)
    assert xg.jit_stats()["launches"] - n0 == 2
    assert fam(last_kernels()) == ["k_reduce_stream", "k_reduce_combine"]
    # the same 8 chunks scattered in memory: chunk by chunk, each chunk's
    # reduction then a merge into the result
    b = fake_chunked((256, 512, 1024), (64, 256, 1024), "float32", spaced=False)
    n0 = xg.jit_stats()["launches"]
    chunked_reduce("sum", b, out=out)
    assert xg.jit_stats()["launches"] - n0 >= 8 + 7
