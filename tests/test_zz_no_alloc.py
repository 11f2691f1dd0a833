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
import json
import os
import subprocess
import sys
import textwrap
from pathlib import Path

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


# A preloaded stand-in for the CUDA runtime's allocation calls: each call is
# counted, then forwarded to the runtime the library loaded.  The library
# reaches the runtime through its shared object (libcudart.so.13), so these
# definitions interpose on every allocation or free it makes.
SHIM = r"""
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stddef.h>
static long g_calls;
long shim_alloc_calls(void) { return g_calls; }
static void *real_sym(const char *name)
{
    void *h = dlopen("libcudart.so.13", RTLD_LAZY | RTLD_NOLOAD);
    return h ? dlsym(h, name) : NULL;
}
#define WRAP(name, params, args) \
    int name params { static int (*real) params; if (!real) real = (int (*) params)real_sym(#name); \
                      ++g_calls; return real ? real args : 999; }
WRAP(cudaMalloc, (void **p, size_t n), (p, n))
WRAP(cudaMallocAsync, (void **p, size_t n, void *s), (p, n, s))
WRAP(cudaMallocFromPoolAsync, (void **p, size_t n, void *pool, void *s), (p, n, pool, s))
WRAP(cudaMallocManaged, (void **p, size_t n, unsigned f), (p, n, f))
WRAP(cudaMallocPitch, (void **p, size_t *pitch, size_t w, size_t h), (p, pitch, w, h))
WRAP(cudaMallocHost, (void **p, size_t n), (p, n))
WRAP(cudaHostAlloc, (void **p, size_t n, unsigned f), (p, n, f))
WRAP(cudaFree, (void *p), (p))
WRAP(cudaFreeAsync, (void *p, void *s), (p, s))
WRAP(cudaFreeHost, (void *p), (p))
"""

CHILD = r"""
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from parallel_distance_oracle_gb300 import graphs as G, pado, _lib
calls = C.CDLL(None).shim_alloc_calls
calls.restype = C.c_long
g = G.rmat(12, 8, 43)
idx = pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=50, batch=512)
ptr = lambda x: x.ctypes.data_as(C.c_void_p)
def q(fn, a, b):
    out = np.full(len(a), 77, np.uint8)
    st = getattr(_lib.lib, fn)(idx._h, len(a), ptr(a), ptr(b), ptr(out))
    return st, out
a1, b1 = (np.ascontiguousarray(x) for x in G.random_pairs(g.n, 262144, 7, distinct=False))
a2, b2 = (np.ascontiguousarray(x) for x in G.random_pairs(g.n, 3000, 8, distinct=False))
warm, _ = q("pado_query_noalloc", a2, b2)      # first call on the device: set-up
c0 = calls()
s1, o1 = q("pado_query_noalloc", a1, b1)
s2, o2 = q("pado_query_noalloc", a2, b2)
c1 = calls()
s3, w1 = q("pado_query", a1, b1)                # the allocating entry point, for contrast
c2 = calls()
print(json.dumps(dict(warm=warm, s1=s1, s2=s2, s3=s3, noalloc_calls=c1 - c0, query_calls=c2 - c1,
                      same=bool(np.array_equal(o1, w1)))))
"""


def test_noalloc_makes_no_allocation_calls(lib, tmp_path):
    """Two calls after the warm-up make no allocation or free call into the
    CUDA runtime (counted by a preloaded stand-in in a child process), while
    pado_query on the same pairs does -- the count sees this library's calls."""
    shim_c, shim = tmp_path / "shim.c", tmp_path / "shim.so"
    shim_c.write_text(SHIM)
    subprocess.run(["gcc", "-shared", "-fPIC", "-O2", "-o", str(shim), str(shim_c), "-ldl"], check=True)
    child = tmp_path / "child.py"
    child.write_text(textwrap.dedent(CHILD))
    repo = str(Path(__file__).resolve().parents[1])
    env = dict(os.environ, LD_PRELOAD=str(shim))
    r = subprocess.run([sys.executable, str(child), repo], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["warm"] == 0 and res["s1"] == 0 and res["s2"] == 0 and res["s3"] == 0, res
    assert res["same"], res
    assert res["noalloc_calls"] == 0, res
    assert res["query_calls"] > 0, res
