"""Batched persistent evaluation against the one-launch-per-instance path
and the oracle.

Tolerances: batched elementwise assignment is bit-exact against xtg_assign
(same operations per element); batched row sums are within 1e-6 * sum|x| of
the FP64 value (compensated FP32) and within that of the per-instance
xtg_reduce result; integer row sums are bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300.batch import Batch, fill_random
from xtensor_gb300.device import DeviceArray, HostArray, Stream
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def instances(n, seed, max_rows=300, max_cols=700):
    g = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        r = int(g.integers(1, max_rows + 1))
        c = int(g.integers(16, max_cols + 1))
        A = g.uniform(-1, 1, (r, c)).astype(np.float32)
        v = g.standard_normal(c).astype(np.float32)
        Cm = g.uniform(-1, 1, (r, c)).astype(np.float32)
        out.append((A, v, Cm))
    return out


def test_batched_row_sums_match_plain_and_oracle():
    xg.init(0)
    data = instances(60, 3)
    dev = [(DeviceArray.from_numpy(A), DeviceArray.from_numpy(v), DeviceArray.from_numpy(Cm)) for A, v, Cm in data]
    outs = [DeviceArray.empty((A.shape[0],), "float32") for A, _, _ in data]
    A0, v0, C0 = dev[0]
    b = Batch(A0 * v0 + C0, reduce="sum")
    for (A, v, Cm), o in zip(dev, outs):
        b.add(A * v + Cm, o)
    b.build(autotune=False)
    b.run()
    info = b.info()
    assert info["instances"] == 60 and info["tiles"] >= 60
    for k, ((A, v, Cm), (dA, dv, dC), o) in enumerate(zip(data, dev, outs)):
        got = o.to_numpy()
        E = (A * v + Cm).astype(np.float64)
        bound = 1e-6 * np.abs(E).sum(1)
        assert (np.abs(got - E.sum(1)) <= bound).all(), k
        plain = ops.reduce("sum", dA * dv + dC, [1]).to_numpy()
        assert (np.abs(got - plain) <= 2 * bound).all(), k
        if k < 3:
            ref = O.reduce("sum", HostArray(A) * HostArray(v) + HostArray(Cm), [1])
            env = np.abs(ref - E.sum(1)) + bound
            assert (np.abs(got - ref) <= env).all()


def test_batched_assign_bit_exact_and_graph_replay():
    xg.init(0)
    data = instances(40, 4, 200, 500)
    dev = [(DeviceArray.from_numpy(A), DeviceArray.from_numpy(v), DeviceArray.from_numpy(Cm)) for A, v, Cm in data]
    outs = [DeviceArray.empty(A.shape, "float32") for A, _, _ in data]
    A0, v0, C0 = dev[0]
    b = Batch(A0 * v0 + xg.exp(-C0))
    for (A, v, Cm), o in zip(dev, outs):
        b.add(A * v + xg.exp(-Cm), o)
    b.build(autotune=False)
    s = Stream()
    b.capture(s)
    assert b.info()["graph_ready"] == 1
    b.replay(s)
    s.sync()
    for (A, v, Cm), (dA, dv, dC), o in zip(data, dev, outs):
        plain = DeviceArray.empty(A.shape, "float32")
        xg.assign(plain, dA * dv + xg.exp(-dC))
        np.testing.assert_array_equal(o.to_numpy(), plain.to_numpy())


def test_batched_int_sums_and_autotune_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("XTG_CACHE_DIR", str(tmp_path))
    xg.init(0)
    g = np.random.default_rng(5)
    arrs = [g.integers(-1000, 1000, (int(g.integers(1, 50)), int(g.integers(16, 300)))).astype(np.int32) for _ in range(30)]
    dev = [DeviceArray.from_numpy(a) for a in arrs]
    outs = [DeviceArray.empty((a.shape[0],), "int64") for a in arrs]
    b = Batch(dev[0], reduce="sum", acc_dtype="int64")
    for d, o in zip(dev, outs):
        b.add(d, o)
    b.build(autotune=True)
    assert b.info()["tuned"] == 1
    b.run()
    for a, o in zip(arrs, outs):
        np.testing.assert_array_equal(o.to_numpy(), a.astype(np.int64).sum(1))
    b2 = Batch(dev[0], reduce="sum", acc_dtype="int64")
    for d, o in zip(dev, outs):
        b2.add(d, o)
    b2.build(autotune=True)
    assert b2.info()["tuned"] == 2  # from the on-disk cache
    assert (tmp_path / "autotune.txt").exists()


@pytest.fixture
def batch_vec():
    def set_(v):
        xg.set_option("batch.vec", v)
    yield set_
    xg.set_option("batch.vec", 1)


@pytest.mark.parametrize("vec", [0, 1])
def test_vector_and_strided_forms(vec, batch_vec):
    """The vector form (16-byte loads where a row's leaves share alignment,
    scalar loads where they do not, scalar head and tail) and the strided
    form: row sums within the compensated bound of FP64, integer sums and
    maxima exact, over ragged widths, rows starting at every alignment
    phase (views offset by one element) and broadcast leaves."""
    batch_vec(vec)
    xg.init(0)
    g = np.random.default_rng(7)
    shapes = [(int(g.integers(1, 90)), int(g.integers(1, 300))) for _ in range(40)] + [(3, 1), (5, 2), (2, 3), (1, 5)]
    # float32: A is a view one element into a wider buffer, so its rows start
    # at other phases than C's
    data, keep = [], []
    for r, c in shapes:
        Abig = g.uniform(-1, 1, (r, c + 3)).astype(np.float32)
        v = g.standard_normal(c).astype(np.float32)
        Cm = g.uniform(-1, 1, (r, c)).astype(np.float32)
        dAbig = DeviceArray.from_numpy(Abig)
        dev = (dAbig[:, 1:c + 1], DeviceArray.from_numpy(v), DeviceArray.from_numpy(Cm))
        keep.append(dAbig)
        data.append((Abig[:, 1:c + 1], v, Cm, dev))
    outs = [DeviceArray.empty((r,), "float32") for r, _ in shapes]
    b = Batch(data[0][3][0] * data[0][3][1] + data[0][3][2], reduce="sum")
    for (_, _, _, (dA, dv, dC)), o in zip(data, outs):
        b.add(dA * dv + dC, o)
    b.build(autotune=False)
    b.run()
    for (A, v, Cm, _), o in zip(data, outs):
        E = A.astype(np.float64) * v + Cm
        assert (np.abs(o.to_numpy() - E.sum(1)) <= 1e-6 * np.abs(E).sum(1) + 1e-30).all()
    # float64 means (two elements per vector)
    xs = [g.standard_normal(sh) for sh in shapes]
    dx = [DeviceArray.from_numpy(x) for x in xs]
    om = [DeviceArray.empty((sh[0],), "float64") for sh in shapes]
    bm = Batch(dx[0], reduce="mean")
    for d, o in zip(dx, om):
        bm.add(d, o)
    bm.build(autotune=False)
    bm.run()
    for x, o in zip(xs, om):
        np.testing.assert_allclose(o.to_numpy(), x.mean(1), rtol=1e-13, atol=1e-15)
    # int32 maxima and uint8 sums (sixteen elements per vector): exact
    ints = [g.integers(-10**6, 10**6, sh).astype(np.int32) for sh in shapes]
    di = [DeviceArray.from_numpy(x) for x in ints]
    oi = [DeviceArray.empty((sh[0],), "int32") for sh in shapes]
    bi = Batch(di[0], reduce="amax")
    for d, o in zip(di, oi):
        bi.add(d, o)
    bi.build(autotune=False)
    bi.run()
    for x, o in zip(ints, oi):
        np.testing.assert_array_equal(o.to_numpy(), x.max(1))
    u8 = [g.integers(0, 256, sh).astype(np.uint8) for sh in shapes]
    du = [DeviceArray.from_numpy(x) for x in u8]
    ou = [DeviceArray.empty((sh[0],), "uint64") for sh in shapes]
    bu = Batch(du[0], reduce="sum", acc_dtype="uint64")
    for d, o in zip(du, ou):
        bu.add(d, o)
    bu.build(autotune=False)
    bu.run()
    for x, o in zip(u8, ou):
        np.testing.assert_array_equal(o.to_numpy(), x.astype(np.uint64).sum(1))


def test_fill_random_is_seeded():
    xg.init(0)
    a = fill_random(DeviceArray.empty((1 << 20,), "float32"), "normal", 0.0, 1.0, 7).to_numpy()
    b = fill_random(DeviceArray.empty((1 << 20,), "float32"), "normal", 0.0, 1.0, 7).to_numpy()
    c = fill_random(DeviceArray.empty((1 << 20,), "float32"), "normal", 0.0, 1.0, 8).to_numpy()
    assert a.tobytes() == b.tobytes() and a.tobytes() != c.tobytes()
    assert abs(a.mean()) < 0.01 and abs(a.std() - 1) < 0.01
    u = fill_random(DeviceArray.empty((1 << 20,), "float32"), "uniform", -1.0, 1.0, 3).to_numpy()
    assert u.min() >= -1 and u.max() < 1
    i = fill_random(DeviceArray.empty((1 << 20,), "int32"), "integers", -(1 << 20), 1 << 20, 2).to_numpy()
    assert i.min() >= -(1 << 20) and i.max() <= (1 << 20)
    ln = fill_random(DeviceArray.empty((1 << 20,), "float32"), "signed_lognormal", 0.0, 2.0, 2).to_numpy()
    assert (ln < 0).mean() > 0.45 and (ln > 0).mean() > 0.45
