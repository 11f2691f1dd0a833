"""Error paths of the GPU library, exercised without faulting or hanging the
GPU (failures are made on the host or by a wait that runs out):

* distance overflow: the reference stores unweighted distances in uint8
  (includes/globals.h:29, 255 = unreachable), so a BFS level of 255 cannot be
  represented; a 300-vertex path labeled with no BP roots reaches it, and both
  the one-graph and the many-graph builders stop with PADO_E_OVERFLOW;
* a grid barrier that never completes: the persistent loops' bounded barrier,
  run by pado_selftest_barrier with one block that never arrives, gives up
  after its limit in every waiting block, and the host sees PADO_E_TIMEOUT;
* a device allocation that fails: pado_debug_fail_alloc makes the n-th
  allocation of a build fail, for every n the build reaches; each such build
  returns PADO_E_NOMEM, hands back no index and releases everything it had
  allocated (pado_debug_live_allocations returns to its value before).
After each failure the device stays usable: a normal build still matches the
oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

E_NOMEM, E_OVERFLOW, E_TIMEOUT = 2, 4, 6


@pytest.fixture(scope="module")
def L(cuda_ok):
    from parallel_distance_oracle_gb300 import _lib
    return _lib


def _a(x, dt):
    return np.ascontiguousarray(x, dt)


def _build_unw(L, g, K, B):
    h = C.c_void_p()
    rank = _a(G.degree_rank(g), np.uint32)
    st = L.lib.pado_unw_build(g.n, L.ptr(_a(g.off, np.uint64)), L.ptr(_a(g.adj, np.uint32)), L.ptr(rank), K, B,
                              C.byref(h))
    return st, h


def _build_w(L, g, B):
    h = C.c_void_p()
    rank = _a(G.degree_rank(g), np.uint32)
    st = L.lib.pado_w_build(g.n, L.ptr(_a(g.off, np.uint64)), L.ptr(_a(g.adj, np.uint32)), L.ptr(_a(g.w, np.uint8)),
                            L.ptr(rank), B, C.byref(h))
    return st, h


def _device_still_labels():
    from parallel_distance_oracle_gb300 import pado
    g = G.rmat(10, 8, 77)
    rank = G.degree_rank(g)
    lab = pado.VertexCentricPLL(g, rank, bp_roots=16, batch=128).export()
    ref = orc.unw_label(g, rank, 16, 128)
    assert np.array_equal(lab.off, ref.off) and np.array_equal(lab.hub, ref.hub)


def test_bfs_level_255_is_an_overflow(L):
    g = G.path_graph(300)
    live = L.lib.pado_debug_live_allocations()
    st, h = _build_unw(L, g, 0, 64)
    assert st == E_OVERFLOW, L.lib.pado_last_error()
    assert not h.value
    assert b"255" in L.lib.pado_last_error()
    assert L.lib.pado_debug_live_allocations() == live
    # a path one level shorter labels fine
    st, h = _build_unw(L, G.path_graph(250), 0, 64)
    assert st == 0, L.lib.pado_last_error()
    L.lib.pado_free(h)
    _device_still_labels()


def test_bfs_level_255_is_an_overflow_in_the_many_graph_build(L):
    from parallel_distance_oracle_gb300 import pado
    gs = [G.rmat(8, 4, 3), G.path_graph(300), G.rmat(7, 4, 4)]
    live = L.lib.pado_debug_live_allocations()
    with pytest.raises(L.PadoError) as ei:
        pado.build_many(gs, bp_roots=0, batch=64)
    assert ei.value.status == E_OVERFLOW
    assert L.lib.pado_debug_live_allocations() == live
    _device_still_labels()


def test_barrier_wait_runs_out(L):
    ret = C.c_uint32(0)
    # one block of eight never arrives: the seven others give up after 2 ms
    st = L.lib.pado_selftest_barrier(8, 3, 2_000_000, C.byref(ret))
    assert st == E_TIMEOUT, L.lib.pado_last_error()
    assert ret.value == 8
    # control: every block arrives and the barrier completes
    st = L.lib.pado_selftest_barrier(8, 8, 2_000_000, C.byref(ret))
    assert st == 0, L.lib.pado_last_error()
    assert ret.value == 8
    _device_still_labels()


def _fail_each_allocation(L, build):
    """Fails allocation n = 1, 2, ... of `build` until a build gets through;
    returns how many allocation points failed."""
    live = L.lib.pado_debug_live_allocations()
    n = 0
    while True:
        n += 1
        assert n < 400, "build never completed"
        L.lib.pado_debug_fail_alloc(n)
        st, h = build()
        L.lib.pado_debug_fail_alloc(0)
        if st == 0:
            L.lib.pado_free(h)
            assert L.lib.pado_debug_live_allocations() == live
            return n - 1
        assert st == E_NOMEM, (n, L.lib.pado_last_error())
        assert not h.value, n
        assert L.lib.pado_debug_live_allocations() == live, n


def test_failed_allocations_release_everything(L):
    import torch
    L.lib.pado_set_scratch_cache(0)
    free0 = torch.cuda.mem_get_info()[0]
    gu = G.rmat(9, 8, 5)
    gw = G.rmat(9, 8, 6, weights=(1, 100))
    nu = _fail_each_allocation(L, lambda: _build_unw(L, gu, 16, 64))
    nw = _fail_each_allocation(L, lambda: _build_w(L, gw, 64))
    assert nu > 10 and nw > 10  # the builds do reach that many allocation points
    L.lib.pado_set_scratch_cache(0)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)
    _device_still_labels()


def test_failed_allocations_in_the_many_graph_build(L):
    from parallel_distance_oracle_gb300 import pado
    gs = [G.rmat(8, 4, 10 + i) for i in range(4)]
    live = L.lib.pado_debug_live_allocations()
    for n in range(1, 400):
        L.lib.pado_debug_fail_alloc(n)
        try:
            idx = pado.build_many(gs, bp_roots=8, batch=64)
        except L.PadoError as e:
            assert e.status == E_NOMEM, (n, str(e))
            assert L.lib.pado_debug_live_allocations() == live, n
            continue
        finally:
            L.lib.pado_debug_fail_alloc(0)
        for x in idx:
            x.close()
        assert n > 10
        break
    assert L.lib.pado_debug_live_allocations() == live
    _device_still_labels()
