""".npy format on the host: the oracle restatement pinned to the reference's
fixtures, and libxtg's header reader / writer (host-only entry points, no
GPU) against the oracle, byte for byte and message for message."""
from __future__ import annotations

import importlib.util
import io
from pathlib import Path

import numpy as np
import pytest

from oracle import npy as N
from xtensor_gb300 import ops
from xtensor_gb300._ffi import XtgError, dtype_code

GOLD = Path(__file__).resolve().parent / "golden" / "npy"
_spec = importlib.util.spec_from_file_location("make_npy_golden", GOLD.parent / "make_npy_golden.py")
G = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(G)

DTYPES = ["bool", "int8", "uint8", "int16", "uint16", "int32", "uint32", "int64", "uint64", "float32", "float64"]


def fixture(stem: str) -> bytes:
    return (GOLD / f"{stem}.le.npy").read_bytes()


@pytest.mark.parametrize("stem", sorted(G.EXPECT))
def test_oracle_loads_reference_fixtures(stem):
    want = G.EXPECT[stem]
    b = fixture(stem)
    layout = "column_major" if "fortran" in stem and want.ndim > 1 else "dynamic"
    got = N.load(b, want.dtype, layout)
    assert got.shape == want.shape
    if want.dtype.kind == "f":  # test_xnpy.cpp compares with isclose (8-digit literals)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-8)
    else:
        np.testing.assert_array_equal(got, want)
    # and numpy agrees with the oracle on every fixture
    np.testing.assert_array_equal(np.load(io.BytesIO(b)), got)


def test_oracle_dump_matches_reference_fixtures():
    """test_xnpy.cpp:125-170: dump_npy(barr) / dump_npy(ularr) are byte-equal
    to bool.le.npy / unsignedlong.le.npy."""
    assert N.dump(G.BOOL) == fixture("bool")
    assert N.dump(G.ULONG) == fixture("unsignedlong")
    # the Fortran fixtures hold the reference's column-major dumps
    assert N.dump(np.asfortranarray(G.BOOL)) == fixture("bool_fortran")
    d = np.load(io.BytesIO(fixture("double")))  # the exact doubles the file holds
    assert N.dump(np.asfortranarray(d)) == fixture("double_fortran")
    assert N.dump(d) == fixture("double")
    assert N.dump(G.INT) == fixture("int")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("shape", [(), (0,), (5,), (3, 4), (2, 0, 3), (2, 3, 4, 5, 1, 2, 3, 2), (123456789, 7)])
@pytest.mark.parametrize("fortran", [False, True])
def test_library_header_writer_is_the_reference_writer(dt, shape, fortran):
    got = ops.npy_format_header(dt, shape, fortran)
    want = N.write_header(N.typestring(dt), fortran, shape)
    assert got == want
    assert len(got) % 64 == 0
    # numpy reads what we write
    descr, f, s, ver, off = N.read_header(got)
    assert (descr, f, s, ver, off) == (N.typestring(dt), fortran, tuple(shape), 1, len(got))
    fake = got + b"\0" * (int(np.prod(shape)) * np.dtype(dt).itemsize if 0 < int(np.prod(shape)) < 1000 else 0)
    if 0 < int(np.prod(shape)) < 1000:
        a = np.load(io.BytesIO(fake))
        assert a.shape == tuple(shape) and a.dtype == np.dtype(dt)


@pytest.mark.parametrize("stem", sorted(G.EXPECT))
def test_library_header_reader_on_fixtures(stem):
    b = fixture(stem)
    h = ops.npy_header(b)
    descr, f, s, ver, off = N.read_header(b)
    assert (h["descr"], h["fortran_order"], h["shape"], h["version"], h["data_offset"]) == (descr, f, s, ver, off)
    assert h["dtype"] == dtype_code(G.EXPECT[stem].dtype)
    assert ops.npy_header(GOLD / f"{stem}.le.npy") == h


def _numpy_file(a, version=None, fortran=False):
    buf = io.BytesIO()
    np.lib.format.write_array(buf, np.asfortranarray(a) if fortran else a, version=version)
    return buf.getvalue()


@pytest.mark.parametrize("version", [(1, 0), (2, 0)])
def test_library_reads_numpy_headers(version):
    """np.save's own spelling (growth padding, version 2.0 length field)."""
    for dt in DTYPES:
        a = np.zeros((4, 3, 2), dtype=dt)
        for fortran in (False, True):
            b = _numpy_file(a, version, fortran)
            h = ops.npy_header(b)
            assert h["version"] == version[0]
            assert h["shape"] == (4, 3, 2) and h["fortran_order"] == fortran
            assert h["descr"] == N.typestring(dt) and h["dtype"] == dtype_code(dt)
            assert h["data_offset"] == len(b) - a.nbytes
            assert N.read_header(b)[:4] == (h["descr"], fortran, (4, 3, 2), version[0])
    # a big-endian file parses; its typestring maps to no device type
    h = ops.npy_header(_numpy_file(np.zeros(3, ">f8")))
    assert h["descr"] == ">f8" and h["dtype"] == -1
    # complex: a valid typestring without a device type
    h = ops.npy_header(_numpy_file(np.zeros(2, np.complex128)))
    assert h["descr"] == "<c16" and h["dtype"] == -1


def _craft(header: str, version=(1, 0), magic=N.MAGIC) -> bytes:
    h = header.encode("latin-1")
    n = 2 if version[0] == 1 else 4
    return magic + bytes(version) + len(h).to_bytes(n, "little") + h


BAD = [
    (_craft("{'descr': '<f8', 'fortran_order': False, 'shape': (3,), }"), "invalid header"),
    (_craft("'descr': '<f8', 'fortran_order': False, 'shape': (3,), }\n"), "unable to unwrap"),
    (_craft("{'fortran_order': False, 'shape': (3,), }\n"), "missing 'descr' key"),
    (_craft("{'descr': '<f8', 'shape': (3,), }\n"), "missing 'fortran_order' key"),
    (_craft("{'descr': '<f8', 'fortran_order': False, }\n"), "missing 'shape' key"),
    (_craft("{'fortran_order': False, 'descr': '<f8', 'shape': (3,), }\n"), "header keys in wrong order"),
    (_craft("{'descr': '<U8', 'fortran_order': False, 'shape': (3,), }\n"), "invalid typestring"),
    (_craft("{'descr': 'f8', 'fortran_order': False, 'shape': (3,), }\n"), "invalid typestring"),
    (_craft("{'descr': '<f8', 'fortran_order': 0, 'shape': (3,), }\n"), "invalid fortran_order value"),
    (_craft("{'descr': '<f8', 'fortran_order': False, 'shape': (3,,4), }\n"), "invalid shape"),
    (_craft("{'descr': '<f8', 'fortran_order': False, 'shape': [3], }\n"), "unable to unwrap"),
    (_craft("{'descr': '<f8', 'fortran_order': False, 'shape': (3,), }\n", version=(3, 0)),
     "unsupported file format version"),
    (_craft("{'descr': '<f8', 'fortran_order': False, 'shape': (3,), }\n", magic=b"\x93NUMPX"),
     "this file do not have a valid npy format."),
    (b"\x93NUM", "io error: failed reading file"),
]


@pytest.mark.parametrize("blob,msg", BAD, ids=[m for _, m in BAD])
def test_header_errors_match_the_reference_messages(blob, msg):
    with pytest.raises(N.NpyError) as eo:
        N.read_header(blob)
    assert str(eo.value) == msg
    with pytest.raises(XtgError) as el:
        ops.npy_header(blob)
    assert el.value.status == 1 and str(el.value).endswith(msg)


def test_oracle_type_and_layout_checks():
    b = fixture("double")
    with pytest.raises(N.NpyError, match="Cast error: formats not matching <f8 vs <f4"):
        N.load(b, np.float32)
    with pytest.raises(N.NpyError, match="layout mismatch"):
        N.load(b, np.float64, "column_major")
    with pytest.raises(N.NpyError, match="layout mismatch"):
        N.load(fixture("double_fortran"), np.float64, "row_major")


def test_missing_file():
    with pytest.raises(XtgError) as e:
        ops.npy_header("/nonexistent/dir/x.npy")
    assert str(e.value).endswith("io error: failed to open a file.")
