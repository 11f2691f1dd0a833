"""Compile the drop-in driver against include/pado_gpu.hpp and libpado_gpu.so."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
PKG = REPO / "parallel_distance_oracle_gb300"


def build(out_dir: Path, sources=None, extra_includes=(), name="dropin") -> Path:
    from parallel_distance_oracle_gb300 import build as gb
    gb.build()
    exe = out_dir / name
    srcs = [str(s) for s in (sources or [HERE / "dropin_main.cpp"])]
    cmd = ["g++", "-std=c++14", "-O2", "-fopenmp", "-w"]
    for inc in extra_includes:
        cmd += ["-I", str(inc)]
    cmd += ["-I", str(REPO / "include")] + srcs + ["-o", str(exe), "-L", str(PKG), "-lpado_gpu",
                                                  f"-Wl,-rpath,{PKG}"]
    subprocess.run(cmd, check=True)
    return exe
