"""Build the CUDA library libpado_gpu.so in-tree, for sm_103a only.

Each translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
a shared library next to this file.  A build is skipped when the library is
newer than every source and header.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = REPO / "include"
# PADO_DEBUG_BOUNDS=1 in the environment selects the bounds-checking build
# (device index checks that record an error word instead of faulting; see
# unw_device.cuh), kept beside the release library under its own name.
DEBUG = os.environ.get("PADO_DEBUG_BOUNDS", "") not in ("", "0")
BUILD = PKG / ("_build_debug" if DEBUG else "_build")
LIB = PKG / ("libpado_gpu_debug.so" if DEBUG else "libpado_gpu.so")
SOURCES = ["capi.cu", "query.cu", "bp.cu", "unw.cu", "unw_many.cu", "weighted.cu", "profile.cu", "noalloc.cu",
           "serve.cu", "ingest.cu", "selftest.cu", "hostcopy.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC),
                     "--expt-relaxed-constexpr"]
    if DEBUG:
        common += ["-DPADO_DEBUG_BOUNDS"]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, "-c", str(CSRC / src), "-o", str(obj)] + common
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-shared", "-o", str(tmp)] + ARCH + [str(o) for o in objs] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
