"""Build libxtg.so (the C ABI + planner + JIT) in-tree, and the C oracle.

Host sources are C++17 compiled by g++; the device templates in
``csrc/xtg_device.cuh`` are embedded into the library as text (NVRTC
instantiates one kernel per expression-tree type at first use, for the
running GPU's arch-specific target, sm_103a on GB300) and are additionally
compiled ahead of time by nvcc for sm_103a (``csrc/xtg_aot.cu``: the kernels
of the standard workloads, and the no-allocation entry points).

Usage: ``python -m xtensor_gb300.build`` or ``build()`` from Python.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
GEN = CSRC / "_gen"
BUILD = PKG / "_build"
LIB = PKG / "lib"
ARCH = os.environ.get("XTG_ARCH", "sm_103a")


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "include" / "cuda.h").exists():
            return Path(cand)
    raise RuntimeError("CUDA toolkit not found (set CUDA_HOME)")


def _lib_dirs(cuda: Path) -> list[Path]:
    dirs = []
    for d in [cuda / "lib64", *sorted((cuda / "targets").glob("*/lib"))]:
        if d.exists():
            dirs.append(d)
    return dirs


def _gen_sources() -> Path:
    GEN.mkdir(parents=True, exist_ok=True)
    out = GEN / "xtg_device_src.h"
    parts = ["// generated by xtensor_gb300/build.py from xtg_params.h and xtg_device.cuh\n#pragma once\n"]
    for var, fname in (("kXtgParamsSrc", "xtg_params.h"), ("kXtgDeviceSrc", "xtg_device.cuh")):
        text = (CSRC / fname).read_text()
        assert ")XTGSRC\"" not in text
        parts.append(f'static const char {var}[] = R"XTGSRC({text})XTGSRC";\n')
    new = "".join(parts)
    if not out.exists() or out.read_text() != new:
        out.write_text(new)
    return out


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stamp(paths: list[Path], extra: str) -> str:
    h = hashlib.sha1(extra.encode())
    for p in paths:
        h.update(p.read_bytes())
    return h.hexdigest()


def build_lib(verbose: bool = False) -> Path:
    cuda = cuda_home()
    _gen_sources()
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{cuda / 'include'}", f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [GEN / "xtg_device_src.h", ROOT / "include" / "xtg.h"]
    cpp = sorted(CSRC.glob("*.cpp"))
    cu = sorted(CSRC.glob("*.cu"))
    nvcc = str(cuda / "bin" / "nvcc")
    jobs = []
    objs = []
    for src in cpp:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        key = _stamp([src, *headers], "g++ -O2")
        stamp = obj.with_suffix(".stamp")
        if obj.exists() and stamp.exists() and stamp.read_text() == key:
            continue
        cmd = ["g++", "-O2", "-g", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", *inc, "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, stamp, key))
    arch_num = ARCH.replace("sm_", "")
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        key = _stamp([src, *headers], f"nvcc {ARCH}")
        stamp = obj.with_suffix(".stamp")
        if obj.exists() and stamp.exists() and stamp.read_text() == key:
            continue
        cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
               f"-gencode=arch=compute_{arch_num},code=sm_{arch_num}", *inc, "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, stamp, key))
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        futs = {ex.submit(_run, cmd): (cmd, stamp, key) for cmd, stamp, key in jobs}
        for f in cf.as_completed(futs):
            cmd, stamp, key = futs[f]
            f.result()
            stamp.write_text(key)
            if verbose:
                print("built", cmd[-1])
    lib = LIB / "libxtg.so"
    ldirs = _lib_dirs(cuda)
    link = ["g++", "-shared", "-o", str(lib), *map(str, objs)]
    for d in ldirs:
        link += [f"-L{d}", f"-Wl,-rpath,{d}"]
        if (d / "stubs").exists():
            link += [f"-L{d / 'stubs'}"]
    link += ["-lcudart", "-lnvrtc", "-lpthread", "-ldl"]
    _run(link)
    return lib


def build_oracle() -> Path:
    """The CPU restatement used by the tests and the CPU baseline only."""
    odir = ROOT / "oracle"
    out = odir / "_build"
    out.mkdir(parents=True, exist_ok=True)
    so = out / "liboracle.so"
    srcs = sorted(odir.glob("*.c"))
    if not srcs:
        return so
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           f"-I{ROOT / 'include'}", *map(str, srcs), "-o", str(so), "-lm"]
    _run(cmd)
    return so


def build(verbose: bool = False) -> None:
    build_lib(verbose)
    build_oracle()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("ok")
