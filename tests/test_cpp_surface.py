"""The C++ xt:: surface: xtensor call sites (tests/cpp/*.cpp, written like the
reference's own tests) compile against include/xtensor/... and run on the GPU
through libxtg."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "test_xt_surface.cpp"


def _compile(out: Path, std: str = "c++20") -> None:
    lib = ROOT / "xtensor_gb300" / "lib"
    cmd = ["g++", f"-std={std}", "-O1", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out), f"-L{lib}", "-lxtg",
           f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


# the reference builds as C++20 (CMakeLists.txt:209); the surface also builds as C++17
@pytest.mark.parametrize("std", ["c++20", "c++17"])
def test_cpp_call_sites_compile(tmp_path, std):
    _compile(tmp_path / "test_xt", std)


@pytest.mark.gpu
def test_cpp_call_sites_run_on_gpu(tmp_path):
    exe = tmp_path / "test_xt"
    _compile(exe, "c++20")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, cwd=tmp_path,
                       env={**os.environ, "XTG_NPY_DIR": str(ROOT / "tests" / "golden" / "npy")})
    print(r.stdout[-6000:])
    assert r.returncode == 0, r.stdout[-6000:] + r.stderr[-2000:]
    assert "0 failed checks" in r.stdout
