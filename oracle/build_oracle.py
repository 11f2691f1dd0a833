"""Build recipe for the test oracle (TEST INFRASTRUCTURE ONLY).

Two products, both git-ignored build outputs:

* ``oracle/liboracle.so`` -- the CPU restatement in ``pado_oracle.cpp``.  Always
  built (here and on the GPU host); the tests, the smoke check and the bench's
  CPU-baseline leg load it through ctypes.
* ``oracle/_ref/libpado_ref_k{50,64}.so`` -- the reference's own labeler
  classes, driven by ``ref_driver.cpp``.  The reference headers do not compile
  with GCC as shipped (missing ``typename`` on dependent constructor calls,
  x86-only intrinsic headers), so ``stage_reference()`` writes a mechanically
  patched copy of the six headers the driver needs into ``oracle/_ref/inc``
  (never committed).  The patches change no algorithm:
    1. ``IndexType::Batch(`` / ``IndexType::DistanceIndexType(`` gain
       ``typename``;
    2. the ``<xmmintrin.h>``/``<immintrin.h>`` includes are dropped (the
       force-included ``ref_prelude.h`` supplies them on x86 and stand-ins
       elsewhere);
    3. the class constant ``BITPARALLEL_SIZE = 50`` becomes the macro
       ``PADO_REF_BP_SIZE`` so that the 64-root configuration can be built;
    4. ``load_index_from_file`` reads the file's root count into a local
       instead of into that constant (pado_unw_unv_unp.h:1194 writes to a
       ``static const`` and faults), so the reference can read index files.
  Staging needs the reference tree (``PADO_REFERENCE_DIR``, default: a
  ``reference`` directory beside the repository); compiling only needs the staged copy, so a host that
  received ``oracle/_ref/inc`` can build the driver without the tree.
* ``oracle/_ref/delete_1_degree`` and ``oracle/_ref/remove_equivalent`` -- the
  reference's two graph-conversion tools (``tools/pseudocode-delete_1-degree_
  vertices.cpp``, ``distributed_version/tools/graph-convert/
  remove_equivalent_vertices.cpp``) compiled unchanged where they lie in the
  reference tree; their headers miss ``<cstdint>`` (and the first ``<cstdio>``/
  ``<cstdlib>``), which the compiler's ``-include`` supplies.  Built only where
  the tree is present: they make the graph-reduction fixtures and pin the
  oracle's reductions in the CPU tests.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REF_OUT = ORACLE_DIR / "_ref"
REF_INC = REF_OUT / "inc"
PORT_SO = ORACLE_DIR / "liboracle.so"

REF_HEADERS = [
    "globals.h",
    "graph.h",
    "pado_unw_unv_unp.h",
    "pado_unw_unv_para.201912311607.parallel_bp_labeling.h",
    "pado_weighted_unv_unp.h",
    "pado_weighted_unv_para.h",
]
REF_BP_SIZES = (50, 64)
# The AVX-512 classes (pado.cpp's `-v 1` modes) and their helper header.
REF_VEC_HEADERS = ["avx512_pado.h", "pado_unw_vec_unp.h", "pado_unw_vec_para.h", "pado_weighted_vec_unp.h",
                   "pado_weighted_vec_para.h"]


def _reference_dir() -> Path:
    return Path(os.environ.get("PADO_REFERENCE_DIR", ORACLE_DIR.parent.parent / "reference"))


def _newer(out: Path, *inputs: Path) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in inputs if p.exists())


def build_port(force: bool = False) -> Path:
    src = ORACLE_DIR / "pado_oracle.cpp"
    if force or not _newer(PORT_SO, src):
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", str(src), "-o", str(PORT_SO)]
        subprocess.run(cmd, check=True)
    return PORT_SO


_TYPENAME_RE = re.compile(r"([^a-zA-Z_:])IndexType::(Batch|DistanceIndexType)\(")


def _patch(text: str) -> str:
    text = _TYPENAME_RE.sub(r"\1typename IndexType::\2(", text)
    text = re.sub(r"^\s*#include\s*<(xmmintrin|immintrin)\.h>\s*$", "", text, flags=re.M)
    text = text.replace("static const inti BITPARALLEL_SIZE = 50;",
                        "static const inti BITPARALLEL_SIZE = PADO_REF_BP_SIZE;")
    # load_index_from_file reads the file's root count into the class constant
    # (a write to read-only storage: it faults); read it into a local instead
    text = text.replace("fin.read((char *) &BITPARALLEL_SIZE, sizeof(BITPARALLEL_SIZE));",
                        "{ inti bp_size_in_file = 0; fin.read((char *) &bp_size_in_file, sizeof(bp_size_in_file)); }")
    return text


REF_DRIVERS = ["pado.cpp", "query_distance.cpp"]


def stage_reference() -> bool:
    """Write the patched header copy into oracle/_ref/inc, and unmodified
    copies of the reference's two drivers into oracle/_ref/drivers (the
    drop-in test builds them against include/pado_gpu.hpp).  False if no
    tree."""
    src = _reference_dir() / "includes"
    if not src.is_dir():
        return False
    REF_INC.mkdir(parents=True, exist_ok=True)
    for name in REF_HEADERS + REF_VEC_HEADERS:
        out = REF_INC / name
        text = _patch((src / name).read_text(errors="replace"))
        if not out.exists() or out.read_text(errors="replace") != text:
            out.write_text(text)
    drv = REF_OUT / "drivers"
    drv.mkdir(parents=True, exist_ok=True)
    for name in REF_DRIVERS:
        text = (_reference_dir() / name).read_text(errors="replace")
        out = drv / name
        if not out.exists() or out.read_text(errors="replace") != text:
            out.write_text(text)
    return True


def ref_so(k: int) -> Path:
    return REF_OUT / f"libpado_ref_k{k}.so"


def build_reference(force: bool = False, sizes=REF_BP_SIZES) -> list[Path]:
    """Compile the reference driver for each BP size.  [] if not staged."""
    stage_reference()
    if not all((REF_INC / h).exists() for h in REF_HEADERS):
        return []
    deps = [ORACLE_DIR / "ref_driver.cpp", ORACLE_DIR / "ref_prelude.h", Path(__file__)] + [REF_INC / h for h in REF_HEADERS]
    procs = []
    outs = []
    for k in sizes:
        out = ref_so(k)
        outs.append(out)
        if not force and _newer(out, *deps):
            continue
        # -fno-gnu-unique: both root-count builds are loaded into one process
        # (ctypes, RTLD_LOCAL); with GNU-unique binding their template static
        # members (BITPARALLEL_SIZE, which store_index_to_file writes) would
        # bind process-wide to whichever library was loaded first
        cmd = ["g++", "-std=c++14", "-O3", "-fopenmp", "-fPIC", "-shared", "-w", "-fno-gnu-unique",
               f"-DPADO_REF_BP_SIZE={k}", "-I", str(REF_INC), "-I", str(ORACLE_DIR),
               str(ORACLE_DIR / "ref_driver.cpp"), "-o", str(out)]
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference driver build failed: " + " ".join(cmd))
    return outs


def vec_so() -> Path:
    return REF_OUT / "libpado_refvec_k50.so"


def host_has_avx512() -> bool:
    """The reference's AVX-512 classes need an x86 CPU with these extensions."""
    try:
        flags = Path("/proc/cpuinfo").read_text()
    except OSError:
        return False
    need = ("avx512f", "avx512bw", "avx512vl", "avx512dq", "avx512cd")
    return all(f" {x}" in flags for x in need)


def build_reference_vec(force: bool = False) -> Path | None:
    """Compile ref_vec_driver.cpp (the reference's AVX-512 labelers, K = 50)
    where the staged headers exist and the CPU has AVX-512; else None."""
    stage_reference()
    if not host_has_avx512() or not all((REF_INC / h).exists() for h in REF_HEADERS[:2] + REF_VEC_HEADERS):
        return None
    out = vec_so()
    deps = [ORACLE_DIR / "ref_vec_driver.cpp", ORACLE_DIR / "ref_prelude.h", Path(__file__)] + \
        [REF_INC / h for h in REF_HEADERS[:2] + REF_VEC_HEADERS]
    if force or not _newer(out, *deps):
        # -fno-strict-aliasing: the AVX-512 classes read vector lanes through
        # casted pointers (`int *tmp_vindex = (int *) &vindex;`,
        # pado_weighted_vec_unp.h:1800), which their intended compiler (icpc)
        # tolerates; GCC's aliasing optimisation turns those reads into
        # garbage indices and the weighted class then writes out of bounds
        cmd = ["g++", "-std=c++14", "-O3", "-fopenmp", "-fPIC", "-shared", "-w", "-fno-gnu-unique",
               "-fno-strict-aliasing", "-mavx512f", "-mavx512bw", "-mavx512vl", "-mavx512dq", "-mavx512cd", "-DPADO_REF_BP_SIZE=50",
               "-I", str(REF_INC), "-I", str(ORACLE_DIR), str(ORACLE_DIR / "ref_vec_driver.cpp"), "-o", str(out)]
        subprocess.run(cmd, check=True)
    return out


REF_TOOLS = {
    "delete_1_degree": ("tools/pseudocode-delete_1-degree_vertices.cpp", [], []),
    "remove_equivalent": ("distributed_version/tools/graph-convert/remove_equivalent_vertices.cpp",
                          ["distributed_version/includes", "includes"], ["-fopenmp"]),
}


def ref_tool(name: str) -> Path:
    return REF_OUT / name


def build_reference_tools(force: bool = False) -> list[Path]:
    """Compile the reference's graph-conversion tools.  [] without the tree."""
    root = _reference_dir()
    outs = []
    for name, (src, incs, extra) in REF_TOOLS.items():
        path = root / src
        if not path.exists():
            return []
        out = ref_tool(name)
        outs.append(out)
        if not force and _newer(out, path):
            continue
        REF_OUT.mkdir(parents=True, exist_ok=True)
        cmd = (["g++", "-std=c++14", "-O2", "-w", "-include", "cstdint", "-include", "cstdio", "-include", "cstdlib"]
               + extra + sum((["-I", str(root / i)] for i in incs), []) + [str(path), "-o", str(out)])
        subprocess.run(cmd, check=True)
    return outs


def build_all() -> None:
    build_port()
    build_reference()
    build_reference_tools()


if __name__ == "__main__":
    build_all()
    print("oracle:", PORT_SO, "reference:", [str(p) for p in build_reference()], file=sys.stderr)
