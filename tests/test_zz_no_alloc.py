"""pado_query_noalloc: queries for callers that cannot let a library allocate
device memory -- serving threads that cannot afford the device-wide stalls
cudaMalloc/cudaFree can cause, and processes whose GPU memory is owned by
another allocator.  It stages pairs and results through a fixed area compiled
into the library instead of allocating; its answers must be exactly those of
pado_query (distances are integers, so the tolerance is zero), call after call,
since successive calls reuse the same area.

This file is named to be collected last, so a run that stops at the first
failure has run every other test already; it also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144  # PADO_NOALLOC_MAX_PAIRS in include/pado_gpu.h


@pytest.fixture(scope="module")
def lib(cuda_ok):
    from parallel_distance_oracle_gb300 import _lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _query(lib, h, fn, a, b, dtype):
    out = np.full(len(a), 77, dtype=dtype)  # poison: every slot must be written
    st = getattr(lib.lib, fn)(h, len(a), _ptr(a), _ptr(b), _ptr(out))
    assert st == 0, lib.lib.pado_last_error().decode()
    return out


def _pairs(n, k, seed):
    a, b = G.random_pairs(n, k, seed, distinct=False)
    a[:16] = n + 3  # out-of-range ids are answered too
    return np.ascontiguousarray(a), np.ascontiguousarray(b)


@pytest.mark.parametrize("weighted", [False, True])
def test_noalloc_matches_pado_query_twice_in_a_row(lib, weighted):
    from parallel_distance_oracle_gb300 import pado
    if weighted:
        g = G.rmat(11, 8, 41, weights=(1, 100))
        idx = pado.WeightedVertexCentricPLL(g, G.degree_rank(g), batch=256)
        dtype = np.int16
    else:
        g = G.rmat(12, 8, 41)
        idx = pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=50, batch=512)
        dtype = np.uint8
    # two different calls in a row: the second must not see the first's data
    for k, seed in ((MAX_PAIRS, 1), (5000, 2)):
        a, b = _pairs(g.n, k, seed)
        want = _query(lib, idx._h, "pado_query", a, b, dtype)
        got = _query(lib, idx._h, "pado_query_noalloc", a, b, dtype)
        assert np.array_equal(got, want)


def test_noalloc_rejects_batches_beyond_its_area(lib):
    from parallel_distance_oracle_gb300 import pado
    g = G.rmat(9, 8, 42)
    idx = pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=16, batch=64)
    a, b = _pairs(g.n, MAX_PAIRS + 1, 3)
    out = np.zeros(len(a), np.uint8)
    st = lib.lib.pado_query_noalloc(idx._h, len(a), _ptr(a), _ptr(b), _ptr(out))
    assert st == 1  # PADO_E_ARG
    assert b"exceed" in lib.lib.pado_last_error()
    # and the entry point still works afterwards
    a, b = _pairs(g.n, 1000, 4)
    assert np.array_equal(_query(lib, idx._h, "pado_query_noalloc", a, b, np.uint8),
                          _query(lib, idx._h, "pado_query", a, b, np.uint8))
