"""C-ABI surface checks that need no GPU: the library loads, exports every
symbol include/pado_gpu.h declares, and rejects bad arguments / files with
status codes before touching the device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from parallel_distance_oracle_gb300 import _lib, graphs as G, pado

HEADER = Path(__file__).resolve().parents[1] / "include" / "pado_gpu.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(pado_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_what_binding_knows():
    assert declared_functions() == sorted(_lib.EXPORTED)


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports_symbol(name):
    assert hasattr(_lib.lib, name)


def test_status_strings():
    assert _lib.lib.pado_status_string(0) == b"ok"
    assert _lib.lib.pado_status_string(1) == b"invalid argument"
    assert b"sm_103a" in _lib.lib.pado_version()


def _build_status(**kw):
    g = kw.pop("g", G.path_graph(6))
    rank = kw.pop("rank", G.degree_rank(g))
    K, B = kw.pop("K", 2), kw.pop("B", 4)
    h = C.c_void_p()
    off = np.ascontiguousarray(g.off, np.uint64)
    adj = np.ascontiguousarray(g.adj, np.uint32)
    rk = None if rank is None else np.ascontiguousarray(rank, np.uint32)
    st = _lib.lib.pado_unw_build(g.n, _lib.ptr(off), _lib.ptr(adj), _lib.ptr(rk), K, B, C.byref(h))
    return st, h


def test_bad_batch_size_rejected():
    assert _build_status(B=0)[0] == 1
    assert _build_status(B=4096)[0] == 1


def test_too_many_bp_roots_rejected():
    assert _build_status(K=65)[0] == 1


def test_bad_offsets_rejected():
    g = G.path_graph(6)
    g.off = g.off.copy()
    g.off[0] = 1
    assert _build_status(g=g)[0] == 1
    assert b"off[0]" in _lib.lib.pado_last_error()
    g = G.path_graph(6)
    g.off = g.off.copy()
    g.off[-1] = 1 << 33
    assert _build_status(g=g)[0] == 1


# Rank permutations and adjacency ids are checked on the device (where the
# CSR is uploaded): tests/test_gpu_parity.py covers them.


def test_missing_index_file_is_io_error(tmp_path):
    h = C.c_void_p()
    assert _lib.lib.pado_load(str(tmp_path / "nope").encode(), 0, C.byref(h)) == 5


def test_truncated_index_file_is_io_error(tmp_path):
    p = tmp_path / "trunc.idx"
    p.write_bytes(np.array([10, 4], np.uint32).tobytes() + b"\x01\x02")
    h = C.c_void_p()
    assert _lib.lib.pado_load(str(p).encode(), 0, C.byref(h)) == 5


def test_python_mirror_raises_pado_error():
    g = G.path_graph(5)
    with pytest.raises(pado.PadoError):
        pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=4, batch=0)
