"""Copy the reference's .npy test fixtures into tests/golden/npy/.

The reference's io tests (test/test_xnpy.cpp) load
test/files/xnpy_files/{double,bool,int,...}{,_fortran}.{le,be}.npy and
compare dump_npy's output byte for byte with bool.le.npy and
unsignedlong.le.npy.  These files are golden data (NumPy's format as the
reference reads and writes it); the GPU machine has no copy of the reference, so
this script copies them next to the tests and checks, with numpy, that each
holds the arrays test_xnpy.cpp expects.

Run (in the build container, where the reference is mounted):
    python tests/golden/make_npy_golden.py <reference checkout>
"""
from __future__ import annotations

import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "npy"

# the arrays test_xnpy.cpp compares the fixtures with
DOUBLE = np.array([
    [[0.29731723, 0.04380157, 0.94748308], [0.85020643, 0.52958618, 0.0598172], [0.77253259, 0.47564231, 0.70274005]],
    [[0.85998447, 0.61160158, 0.44432939], [0.25506765, 0.97420976, 0.15455842], [0.05873659, 0.66191764, 0.01448838]],
    [[0.175919, 0.13850365, 0.94059426], [0.79941809, 0.5124432, 0.51364796], [0.25721979, 0.41608858, 0.06255319]],
])
BOOL = np.array([
    [[0, 0, 1], [1, 1, 0], [1, 0, 1]],
    [[1, 1, 0], [0, 1, 0], [0, 1, 0]],
    [[0, 0, 1], [1, 1, 1], [0, 0, 0]],
], dtype=bool)
INT = np.array([3, 4, 5, 6, 7], dtype=np.int32)
ULONG = np.array([12, 14, 16, 18, 1234321], dtype=np.uint64)

EXPECT = {
    "double": DOUBLE, "double_fortran": DOUBLE,
    "bool": BOOL, "bool_fortran": BOOL,
    "int": INT,
    "unsignedlong": ULONG, "unsignedlong_fortran": ULONG,
}


def main(ref_root: str) -> None:
    src = Path(ref_root) / "test" / "files" / "xnpy_files"
    OUT.mkdir(exist_ok=True)
    for stem, want in EXPECT.items():
        for end in ("le", "be"):
            f = src / f"{stem}.{end}.npy"
            a = np.load(f)
            assert a.shape == want.shape, (f, a.shape)
            if a.dtype.kind == "f":
                assert np.allclose(a, want), f
            else:
                assert (a == want).all(), f
            assert a.dtype.newbyteorder("=") == want.dtype.newbyteorder("=") or a.dtype.kind == "b", (f, a.dtype)
            shutil.copyfile(f, OUT / f.name)
    print(f"wrote {len(list(OUT.glob('*.npy')))} fixtures to {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
