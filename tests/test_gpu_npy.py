"""xt::load_npy / xt::dump_npy through libxtg on the GPU: the reference's
fixtures (tests/golden/npy), numpy round trips of every dtype and order,
strided destinations and sources, the multi-threaded chunk ring at sizes
beyond one chunk, and the reference's error cases.  Every comparison is
bit-exact (the bytes are moved, never converted)."""
from __future__ import annotations

import ctypes as C
import importlib.util
import io
from pathlib import Path

import numpy as np
import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import ops
from xtensor_gb300._ffi import XtgError, lib
from xtensor_gb300.batch import fill_random
from xtensor_gb300.device import DeviceArray
from oracle import npy as N

from util import rng

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "npy"
_spec = importlib.util.spec_from_file_location("make_npy_golden", GOLD.parent / "make_npy_golden.py")
G = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(G)

DTYPES = ["bool", "int8", "uint8", "int16", "uint16", "int32", "uint32", "int64", "uint64", "float32", "float64"]


@pytest.fixture
def chunk():
    def set_(nbytes, threads=None):
        xg.set_option("npy.chunk_bytes", nbytes)
        if threads is not None:
            xg.set_option("npy.threads", threads)
    yield set_
    xg.set_option("npy.chunk_bytes", -1)
    xg.set_option("npy.threads", -1)


def _bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint8).reshape(-1)


def _random(shape, dt, g):
    if dt == "bool":
        return g.random(shape) < 0.5
    if dt.startswith("float"):
        return g.standard_normal(shape).astype(dt)
    info = np.iinfo(dt)
    return g.integers(info.min, info.max, shape, dtype=dt, endpoint=True)


@pytest.mark.parametrize("stem", sorted(G.EXPECT))
def test_reference_fixtures_load(stem):
    """test_xnpy.cpp:39-83: the fixtures load as the arrays the test expects
    (equal to the oracle's reading, bit for bit)."""
    path = GOLD / f"{stem}.le.npy"
    want = N.load(path.read_bytes(), G.EXPECT[stem].dtype)
    for src in (path, path.read_bytes()):
        d = ops.load_npy(src, G.EXPECT[stem].dtype)
        got = d.to_numpy()
        assert got.shape == want.shape
        np.testing.assert_array_equal(_bits(got), _bits(want))
    if "fortran" in stem and want.ndim > 1:
        d = ops.load_npy(path, layout="column_major")
        assert d.strides == (1, 3, 9)  # a column-major result, as the reference's dynamic layout
        with pytest.raises(XtgError, match="layout mismatch between npy file and requested layout"):
            ops.load_npy(path, layout="row_major")
    elif want.ndim > 1:
        with pytest.raises(XtgError, match="layout mismatch between npy file and requested layout"):
            ops.load_npy(path, layout="column_major")


def test_reference_fixtures_dump_bytes(tmp_path):
    """test_xnpy.cpp:125-170: dump_npy of the bool and uint64 arrays equals the
    fixtures byte for byte (file and in-memory forms)."""
    for arr, stem in ((G.BOOL, "bool"), (G.ULONG, "unsignedlong"), (G.INT, "int")):
        fixture = (GOLD / f"{stem}.le.npy").read_bytes()
        d = DeviceArray.from_numpy(arr)
        f = tmp_path / f"{stem}.npy"
        ops.dump_npy(f, d)
        assert f.read_bytes() == fixture
        assert ops.dump_npy(d) == fixture
        back = ops.load_npy(f, arr.dtype).to_numpy()
        np.testing.assert_array_equal(back, arr)
    # a column-major device array writes a Fortran-order file (the reference's
    # eval of a column_major container)
    d = ops.load_npy(GOLD / "double_fortran.le.npy")
    assert ops.dump_npy(d) == (GOLD / "double_fortran.le.npy").read_bytes()


@pytest.mark.parametrize("dt", DTYPES)
def test_numpy_round_trips(dt, tmp_path):
    g = rng(41)
    for shape in [(), (0,), (1,), (7,), (33, 65), (3, 0, 5), (5, 17, 19), (2, 3, 2, 3, 2, 3, 2, 3)]:
        a = _random(shape, dt, g)
        for fortran in (False, True):
            f = tmp_path / "a.npy"
            # (np.asfortranarray makes a 0-d array 1-d)
            np.save(f, np.asfortranarray(a) if fortran and a.ndim else a)
            d = ops.load_npy(f)
            assert d.dtype == xg.dtype_code(dt) and d.shape == a.shape
            np.testing.assert_array_equal(_bits(d.to_numpy()), _bits(a))
            # into a row-major destination: reordered on the device
            out = DeviceArray.empty(a.shape, dt)
            ops.load_npy(f, dt, out=out)
            np.testing.assert_array_equal(_bits(out.to_numpy()), _bits(a))
            # and written back: numpy reads the same values, the bytes are the oracle's dump
            ops.dump_npy(f, d)
            np.testing.assert_array_equal(np.load(f), a)
            assert f.read_bytes() == N.dump(np.asfortranarray(a) if fortran and a.ndim > 1 else a)


def test_strided_destination_and_source(tmp_path):
    g = rng(42)
    a = g.standard_normal((40, 50, 60))
    f = tmp_path / "a.npy"
    np.save(f, a)
    # destination is a transposed view of a bigger buffer
    big = DeviceArray.empty((60, 50, 40), "float64")
    dst = big.transpose((2, 1, 0))
    ops.load_npy(f, "float64", out=dst)
    np.testing.assert_array_equal(big.to_numpy(), a.transpose(2, 1, 0))
    # destination every other element
    buf = DeviceArray.empty((40, 50, 120), "float64")
    ops.load_npy(f, "float64", out=buf[:, :, ::2])
    np.testing.assert_array_equal(buf.to_numpy()[:, :, ::2], a)
    # source: a strided view and an expression are evaluated first (C order)
    d = DeviceArray.from_numpy(a)
    v = d[::2, :, 5:45:3]
    ops.dump_npy(f, v)
    assert f.read_bytes() == N.dump(np.ascontiguousarray(a[::2, :, 5:45:3]))
    e = d * 2.0 + 1.0
    ops.dump_npy(f, e)
    np.testing.assert_array_equal(np.load(f), a * 2.0 + 1.0)


@pytest.mark.parametrize("chunk_bytes,threads", [(1 << 16, 1), (1 << 16, 3), (1 << 20, 8), (8 << 20, 8)])
def test_chunk_ring_many_chunks(chunk_bytes, threads, chunk, tmp_path):
    """Sizes that are not multiples of the chunk: every chunk lands where it
    belongs, for any number of host threads."""
    chunk(chunk_bytes, threads)
    g = rng(43)
    a = g.standard_normal((3, 1000, 1777)).astype(np.float32)  # 21.3 MB
    f = tmp_path / "a.npy"
    np.save(f, a)
    d = ops.load_npy(f)
    np.testing.assert_array_equal(_bits(d.to_numpy()), _bits(a))
    f2 = tmp_path / "b.npy"
    ops.dump_npy(f2, d)
    assert f2.read_bytes() == N.dump(a)
    # in memory, pageable buffer
    img = f.read_bytes()
    d2 = ops.load_npy(img)
    np.testing.assert_array_equal(_bits(d2.to_numpy()), _bits(a))
    assert ops.dump_npy(d2) == N.dump(a)


def test_pinned_buffer_direct_path():
    g = rng(44)
    a = g.integers(-1000, 1000, (257, 1031)).astype(np.int64)
    img = N.dump(a)
    p = C.c_void_p()
    assert lib().xtg_host_alloc(C.byref(p), len(img)) == 0
    try:
        C.memmove(p.value, img, len(img))
        out = DeviceArray.empty(a.shape, "int64")
        arr = out.xtg_array()
        assert lib().xtg_npy_load_buffer(p, len(img), C.byref(arr), 0, None) == 0
        np.testing.assert_array_equal(out.to_numpy(), a)
        # and saved into the same pinned buffer
        C.memset(p.value, 0, len(img))
        n = C.c_size_t()
        assert lib().xtg_npy_save_buffer(C.byref(arr), p, len(img), C.byref(n), None) == 0
        assert n.value == len(img)
        assert C.string_at(p.value, len(img)) == img
    finally:
        lib().xtg_host_free(p)


def test_large_round_trip(tmp_path):
    """2^26 float32 (256 MiB): through the file, checksums of the bytes."""
    n = 1 << 26
    d = DeviceArray.empty((n,), "float32")
    fill_random(d, "normal", 0.0, 1.0, 7)
    f = tmp_path / "big.npy"
    ops.dump_npy(f, d)
    host = d.to_numpy()
    assert f.stat().st_size == 128 + 4 * n
    np.testing.assert_array_equal(np.load(f, mmap_mode="r")[::4099], host[::4099])
    back = ops.load_npy(f)
    s_dev = ops.reduce("sum", back.reshape((n,)), acc_dtype="float64").to_numpy()
    s_ref = ops.reduce("sum", d, acc_dtype="float64").to_numpy()
    assert s_dev == s_ref
    np.testing.assert_array_equal(_bits(back.to_numpy()), _bits(host))


def test_errors(tmp_path):
    f = tmp_path / "d.npy"
    a = np.arange(12.0).reshape(3, 4)
    np.save(f, a)
    with pytest.raises(XtgError, match="Cast error: formats not matching <f8 vs <f4"):
        ops.load_npy(f, "float32")
    with pytest.raises(XtgError) as e:
        ops.load_npy(f, "float64", out=DeviceArray.empty((4, 3), "float64"))
    assert e.value.status == 5
    fb = tmp_path / "be.npy"
    np.save(fb, a.astype(">f8"))
    with pytest.raises(XtgError, match="Cast error: formats not matching >f8"):
        ops.load_npy(fb)
    with pytest.raises(XtgError, match="Cast error: formats not matching >f8 vs <f8"):
        ops.load_npy(fb, "float64")
    with pytest.raises(XtgError, match="io error: failed to open a file."):
        ops.load_npy(tmp_path / "missing.npy", "float64")
    # truncated data
    ft = tmp_path / "t.npy"
    ft.write_bytes(f.read_bytes()[:-8])
    with pytest.raises(XtgError, match="io error: failed reading file"):
        ops.load_npy(ft, "float64")
    with pytest.raises(XtgError, match="io error: failed reading file"):
        ops.load_npy(ft.read_bytes(), "float64")
    # bfloat16 has no npy typestring
    with pytest.raises(XtgError) as e:
        ops.dump_npy(tmp_path / "x.npy", DeviceArray.empty((3,), "bfloat16"))
    assert e.value.status == 9
    # unwritable path
    with pytest.raises(XtgError, match="IO Error: failed to open file"):
        ops.dump_npy(tmp_path / "no" / "dir" / "x.npy", DeviceArray.from_numpy(a))


@pytest.mark.parametrize("where", ["/dev/shm", None])
def test_save_paths_by_file_system(where, tmp_path):
    """tmpfs: the file is mapped and filled by every thread; other file
    systems: one writer in file order.  Both give the oracle's bytes."""
    import os
    import tempfile
    if where is not None and not os.path.isdir(where):
        pytest.skip(f"{where} absent")
    d = Path(tempfile.mkdtemp(dir=where)) if where else tmp_path
    try:
        g = rng(46)
        for shape in ((3, 1000, 1777), (1 << 18,), (64, 64)):  # 21 MB, 1 MiB, 16 KiB
            a = g.standard_normal(shape).astype(np.float32)
            f = d / "s.npy"
            f.write_bytes(b"x" * (3 * a.nbytes))  # truncated on open
            ops.dump_npy(f, DeviceArray.from_numpy(a))
            assert f.read_bytes() == N.dump(a)
            np.testing.assert_array_equal(_bits(ops.load_npy(f).to_numpy()), _bits(a))
    finally:
        if where:
            import shutil
            shutil.rmtree(d, ignore_errors=True)
