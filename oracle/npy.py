"""Restatement of the reference's .npy reader and writer — test infrastructure only.

Follows include/xtensor/io/xnpy.hpp:
  * build_typestring (xnpy.hpp:77-188): endianness char ('|' for one-byte
    types), kind letter, item size;
  * parse_header (xnpy.hpp:237-390): strip the '\\n', remove every space,
    unwrap the {...}, find the three keys in order, check the typestring
    against '([<>|])([ifucb])(\\d+)', 'True'/'False', a comma list in (...);
  * write_header (xnpy.hpp:394-463): the dict spelled
    "{'descr': '<f8', 'fortran_order': False, 'shape': (3, 3, 3), }",
    padded with 64 - (metadata_len % 64) spaces, then '\\n'; version 2.0 once
    the version 1.0 metadata would reach 255 * 255 bytes;
  * load_npy_file / cast_impl (xnpy.hpp:540-700): version 1.0 / 2.0 only,
    the typestring and layout checks with the reference's messages.
Pinned against the reference's fixtures (tests/golden/npy/, copied by
tests/golden/make_npy_golden.py) in tests/test_oracle_npy.py.
"""
from __future__ import annotations

import re
import sys

import numpy as np

MAGIC = b"\x93NUMPY"


class NpyError(RuntimeError):
    pass


def typestring(dtype) -> str:
    dt = np.dtype(dtype)
    kind = {"b": "b", "i": "i", "u": "u", "f": "f", "c": "c"}[dt.kind]
    end = "|" if dt.itemsize <= 1 else ("<" if sys.byteorder == "little" else ">")
    return f"{end}{kind}{dt.itemsize}"


def write_header(descr: str, fortran_order: bool, shape) -> bytes:
    s_shape = "(" + "".join(f"{d}, " for d in shape)
    if len(shape) > 1:
        s_shape = s_shape[:-2]
    elif len(shape) == 1:
        s_shape = s_shape[:-1]
    s_shape += ")"
    d = f"{{'descr': '{descr}', 'fortran_order': {'True' if fortran_order else 'False'}, 'shape': {s_shape}, }}"
    pre = len(d) + 1
    meta = 6 + 2 + 2 + pre
    ver = 1
    if meta >= 255 * 255:
        meta = 6 + 2 + 4 + pre
        ver = 2
    d = d + " " * (64 - meta % 64) + "\n"
    hl = len(d).to_bytes(2 if ver == 1 else 4, "little")
    return MAGIC + bytes([ver, 0]) + hl + d.encode("latin-1")


def _unwrap(s: str, a: str, b: str) -> str:
    if len(s) >= 2 and s[0] == a and s[-1] == b:
        return s[1:-1]
    raise NpyError("unable to unwrap")


def parse_header(header: str):
    if not header.endswith("\n"):
        raise NpyError("invalid header")
    h = _unwrap(header[:-1].replace(" ", ""), "{", "}")
    kd, kf, ks = h.find("'descr'"), h.find("'fortran_order'"), h.find("'shape'")
    if kd < 0:
        raise NpyError("missing 'descr' key")
    if kf < 0:
        raise NpyError("missing 'fortran_order' key")
    if ks < 0:
        raise NpyError("missing 'shape' key")
    if not (kd < kf < ks):
        raise NpyError("header keys in wrong order")

    def val(kv: str) -> str:
        kv = kv[:-1] if kv.endswith(",") else kv
        c = kv.find(":")
        return "" if c < 0 else kv[c + 1:]

    descr_s, fortran_s, shape_s = val(h[kd:kf]), val(h[kf:ks]), val(h[ks:])
    if not re.fullmatch(r"'([<>|])([ifucb])(\d+)'", descr_s):
        raise NpyError("invalid typestring")
    if fortran_s == "True":
        fortran = True
    elif fortran_s == "False":
        fortran = False
    else:
        raise NpyError("invalid fortran_order value")
    body = _unwrap(shape_s, "(", ")")
    toks = body.split(",")
    shape = []
    for i, t in enumerate(toks):
        if t == "":
            if i != len(toks) - 1:
                raise NpyError("invalid shape")
        else:
            if not t.isdigit():
                raise NpyError("invalid shape")
            shape.append(int(t))
    return descr_s[1:-1], fortran, tuple(shape)


def read_header(buf: bytes):
    """(descr, fortran_order, shape, version, data_offset) of a file image."""
    if len(buf) < 8:
        raise NpyError("io error: failed reading file")
    if buf[:6] != MAGIC:
        raise NpyError("this file do not have a valid npy format.")
    ver = (buf[6], buf[7])
    if ver == (1, 0):
        n = 2
    elif ver == (2, 0):
        n = 4
    else:
        raise NpyError("unsupported file format version")
    hl = int.from_bytes(buf[8:8 + n], "little")
    start = 8 + n
    descr, fortran, shape = parse_header(buf[start:start + hl].decode("latin-1"))
    return descr, fortran, shape, ver[0], start + hl


def load(buf: bytes, dtype, layout: str = "dynamic") -> np.ndarray:
    """load_npy<T, L> of a file image: T = dtype, L in dynamic / row_major / column_major."""
    descr, fortran, shape, _, off = read_header(buf)
    want = typestring(dtype)
    if descr != want:
        raise NpyError(f"Cast error: formats not matching {descr} vs {want}")
    if (layout == "column_major" and not fortran) or (layout == "row_major" and fortran):
        raise NpyError("Cast error: layout mismatch between npy file and requested layout.")
    n = int(np.prod(shape, dtype=np.int64)) if shape else 1
    data = np.frombuffer(buf, dtype=np.dtype(dtype), count=n, offset=off)
    return data.reshape(shape, order="F" if fortran else "C")


def dump(a: np.ndarray) -> bytes:
    """dump_npy(e) of a host array: Fortran order for a column-major array of
    rank > 1 (an evaluated column_major container), C order otherwise."""
    fortran = a.ndim > 1 and a.flags.f_contiguous and not a.flags.c_contiguous
    body = np.asfortranarray(a) if fortran else np.ascontiguousarray(a)
    return write_header(typestring(a.dtype), fortran, a.shape) + body.tobytes(order="F" if fortran else "C")
