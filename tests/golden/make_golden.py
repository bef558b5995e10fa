"""Extract golden vectors from the reference's own tests into JSON fixtures.

The reference generates its extended reducer tests with numpy
(test/files/preprocess.py runs the `/*py ... */` blocks of
test/files/cppy_source/*.cppy and writes the arrays, printed with 16
digits, into test/test_extended_*.cpp).  This script reads the generated
C++ file as text and writes the arrays it holds for the reducers on the hot
path to tests/golden/*.json, so that the tests (and the GPU machine, which has no
copy of the reference) can pin the oracle and the GPU path to them.

Run (in the build container, where the reference is mounted):
    python tests/golden/make_golden.py <reference checkout>
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _block(text: str, start: int) -> tuple[str, int]:
    """The balanced {...} block starting at text[start] == '{'."""
    depth = 0
    for i in range(start, len(text)):
        c = text[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return text[start:i + 1], i + 1
    raise ValueError("unbalanced braces")


def _to_list(block: str):
    js = block.replace("{", "[").replace("}", "]")
    js = re.sub(r"\s+", "", js)
    return json.loads(js)


def extract_test(text: str, test_name: str) -> dict:
    """All `xarray<double> py_x = {...};` and `double py_x = v;` inside TEST(..., test_name)."""
    m = re.search(r"TEST\(\s*\w+\s*,\s*" + re.escape(test_name) + r"\s*\)", text)
    if not m:
        raise KeyError(test_name)
    body_start = text.index("{", m.end())
    body, _ = _block(text, body_start)
    line0 = text[: m.start()].count("\n") + 1
    out = {"_source_line": line0}
    for mm in re.finditer(r"xarray<double>\s+(py_\w+)\s*=\s*\{", body):
        blk, _ = _block(body, mm.end() - 1)
        out[mm.group(1)] = _to_list(blk)
    for mm in re.finditer(r"\bdouble\s+(py_\w+)\s*=\s*([-+0-9.eE]+)\s*;", body):
        out[mm.group(1)] = float(mm.group(2))
    return out


def main(ref_root: str) -> None:
    src = Path(ref_root) / "test" / "test_extended_xmath_reducers.cpp"
    text = src.read_text()
    var_std = extract_test(text, "var_std")
    average = extract_test(text, "average")
    fixture = {
        "source": "test/test_extended_xmath_reducers.cpp",
        "generated_by": "test/files/preprocess.py (numpy, 16 significant digits)",
        "var_std": {
            "source_line": var_std["_source_line"],
            "numpy": {"a": "np.random.random(4*5*6*7).reshape(4,5,6,7)", "vr_all": "np.var(a)", "vr_all_ddof": "np.var(a, ddof=1)",
                      "st_all": "np.std(a)", "vr": "np.var(a, axis=(0,2))", "vr_ddof": "np.var(a, axis=(0,2), ddof=1)",
                      "st": "np.std(a, axis=(0,2))"},
            **{k[3:]: v for k, v in var_std.items() if k.startswith("py_")},
        },
        "average": {
            "source_line": average["_source_line"],
            "numpy": {"av": "np.average(a, weights=w, axis=(0,1))"},
            **{k[3:]: v for k, v in average.items() if k.startswith("py_")},
        },
    }
    out = HERE / "xmath_reducers.json"
    out.write_text(json.dumps(fixture, separators=(",", ":")))
    print("wrote", out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
