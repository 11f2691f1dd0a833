"""GPU parity: labels built by the CUDA library are byte-identical to the
reference's (golden fixtures) and to the oracle on fresh seeded graphs, and
every query answer equals the reference's query_distance and BFS/Dijkstra.
Integer work: the bar is bit-exact everywhere."""
import os

import numpy as np
import pytest

from conftest import golden_cases
from helpers import assert_same_unw, assert_same_w, golden_unw_labels, golden_w_labels, load_golden
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


def gpu_unw(pado, g, rank, K, B):
    idx = pado.VertexCentricPLL(g, rank, bp_roots=K, batch=B)
    lab = idx.export()
    return idx, orc.UnwLabels(lab.n, K, lab.off, lab.hub, lab.dist,
                              lab.bpd if K else np.zeros(0, np.uint8), lab.bps if K else np.zeros(0, np.uint64))


def gpu_w(pado, g, rank, B):
    idx = pado.WeightedVertexCentricPLL(g, rank, batch=B)
    lab = idx.export()
    return idx, orc.WLabels(lab.n, lab.off, lab.hub, lab.dist)


@pytest.mark.parametrize("path", golden_cases("unw"), ids=lambda p: p.stem)
def test_unweighted_golden(pado, path):
    z, g = load_golden(path)
    idx, lab = gpu_unw(pado, g, z["rank"], int(z["K"]), int(z["B"]))
    assert_same_unw(lab, golden_unw_labels(z), path.stem)
    assert np.array_equal(idx.query(z["qa"], z["qb"]), z["qd"])


@pytest.mark.parametrize("path", golden_cases("w"), ids=lambda p: p.stem)
def test_weighted_golden(pado, path):
    z, g = load_golden(path)
    idx, lab = gpu_w(pado, g, z["rank"], int(z["B"]))
    assert_same_w(lab, golden_w_labels(z), path.stem)
    assert np.array_equal(idx.query(z["qa"], z["qb"]), z["qd"])


UNW_CASES = [
    ("rmat", 11, 8, 1, 50, 256), ("rmat", 11, 16, 2, 64, 64), ("rmat", 12, 8, 3, 16, 1024), ("rmat", 10, 8, 4, 0, 100),
    ("rmat", 10, 4, 5, 64, 33), ("er", 3000, 6, 6, 50, 512), ("grid", 3000, 0, 7, 50, 128), ("rmat", 9, 8, 8, 8, 1),
    ("rmat", 10, 8, 9, 50, 2048),
]


def make_graph(kind, a, b, seed, weights=None):
    if kind == "rmat":
        return G.rmat(a, b, seed, weights=weights)
    if kind == "er":
        g = G.erdos_renyi(a, b, seed)
    else:
        g = G.grid_with_shortcuts(a, 0.02, seed)
    if weights:
        src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
        dst = g.adj.astype(np.int64)
        key = np.minimum(src, dst) * g.n + np.maximum(src, dst)
        u, inv = np.unique(key, return_inverse=True)
        g.w = np.random.Generator(np.random.PCG64(seed)).integers(weights[0], weights[1] + 1, len(u))[inv].astype(np.uint8)
    return g


@pytest.mark.parametrize("case", UNW_CASES, ids=lambda c: "-".join(map(str, c)))
def test_unweighted_vs_oracle(pado, case):
    kind, a, b, seed, K, B = case
    g = make_graph(kind, a, b, seed)
    rank = G.degree_rank(g)
    idx, lab = gpu_unw(pado, g, rank, K, B)
    ref = orc.unw_label(g, rank, K, B)
    assert_same_unw(lab, ref, str(case))
    qa, qb = G.random_pairs(g.n, 20000, seed + 7)
    assert np.array_equal(idx.query(qa, qb), orc.unw_query(ref, qa, qb))


W_CASES = [("rmat", 11, 8, 1, 512, (1, 100)), ("rmat", 11, 8, 2, 64, (1, 7)), ("rmat", 10, 16, 3, 1024, (1, 100)),
           ("er", 2000, 6, 4, 256, (1, 20)), ("grid", 2000, 0, 5, 100, (1, 5)), ("rmat", 9, 8, 6, 1, (1, 100)),
           ("rmat", 10, 8, 7, 2048, (1, 100))]


@pytest.mark.parametrize("case", W_CASES, ids=lambda c: "-".join(map(str, c[:5])))
def test_weighted_vs_oracle(pado, case):
    kind, a, b, seed, B, wr = case
    g = make_graph(kind, a, b, seed, weights=wr)
    rank = G.degree_rank(g)
    idx, lab = gpu_w(pado, g, rank, B)
    ref = orc.w_label(g, rank, B)
    assert_same_w(lab, ref, str(case))
    qa, qb = G.random_pairs(g.n, 20000, seed + 7)
    assert np.array_equal(idx.query(qa, qb), orc.w_query(ref, qa, qb))


def test_c1_config_parity_and_bfs(pado):
    """R-MAT s14/ef8, degree order, K=50, B=1024; 100k queries."""
    g = G.rmat(14, 8, 1)
    rank = G.degree_rank(g)
    idx, lab = gpu_unw(pado, g, rank, 50, 1024)
    ref = orc.unw_label(g, rank, 50, 1024)
    assert_same_unw(lab, ref, "C1")
    qa, qb = G.random_pairs(g.n, 100000, 11)
    q = idx.query(qa, qb)
    assert np.array_equal(q, orc.unw_query(ref, qa, qb))
    for i in range(0, 100000, 2500):
        assert q[i] == orc.bfs(g, int(qa[i]))[qb[i]]


def test_weighted_queries_equal_dijkstra(pado):
    g = G.rmat(12, 8, 3, weights=(1, 100))
    idx, _ = gpu_w(pado, g, G.degree_rank(g), 512)
    qa, qb = G.random_pairs(g.n, 2000, 13)
    q = idx.query(qa, qb)
    for i in range(0, 2000, 50):
        assert q[i] == orc.dijkstra(g, int(qa[i]))[qb[i]]


def test_ranked_build_then_order_labels(pado):
    g = G.rmat(10, 8, 12)
    rank = G.degree_rank(g)
    idx1, lab1 = gpu_unw(pado, g, rank, 50, 128)
    # relabel on the host the way Graph::id_transfer does, then build ranked
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    rg = G.csr_from_edges(g.n, rank[src].astype(np.int64), rank[g.adj].astype(np.int64))
    idx2 = pado.VertexCentricPLL(rg, None, bp_roots=50, batch=128)
    idx2.order_labels(rank=rank)
    l2 = idx2.export()
    assert np.array_equal(l2.hub, lab1.hub) and np.array_equal(l2.off, lab1.off)
    qa, qb = G.random_pairs(g.n, 5000, 3)
    assert np.array_equal(idx1.query(qa, qb), idx2.query(qa, qb))


def test_store_format_matches_oracle_and_loads(pado, tmp_path):
    g = G.rmat(10, 8, 13)
    rank = G.degree_rank(g)
    idx, _ = gpu_unw(pado, g, rank, 50, 256)
    p1 = tmp_path / "gpu.idx"
    idx.store_index_to_file(str(p1))
    lib = orc.port()
    h = lib.orc_unw_build(g.n, np.ascontiguousarray(g.off, np.uint64), np.ascontiguousarray(g.adj, np.uint32),
                          np.ascontiguousarray(rank, np.uint32), 50, 256)
    p2 = tmp_path / "orc.idx"
    assert lib.orc_unw_store(h, str(p2).encode()) == 0
    lib.orc_unw_free(h)
    assert p1.read_bytes() == p2.read_bytes()
    idx2 = pado.VertexCentricPLL()
    idx2.load_index_from_file(str(p1))
    qa, qb = G.random_pairs(g.n, 5000, 5)
    assert np.array_equal(idx.query(qa, qb), idx2.query(qa, qb))


def test_weighted_store_load(pado, tmp_path):
    g = G.rmat(10, 8, 14, weights=(1, 100))
    rank = G.degree_rank(g)
    idx, _ = gpu_w(pado, g, rank, 128)
    p = tmp_path / "w.idx"
    idx.store_index_to_file(str(p))
    lib = orc.port()
    h = lib.orc_w_build(g.n, np.ascontiguousarray(g.off, np.uint64), np.ascontiguousarray(g.adj, np.uint32),
                        np.ascontiguousarray(g.w, np.uint8), np.ascontiguousarray(rank, np.uint32), 128, 0)
    p2 = tmp_path / "orc.idx"
    assert lib.orc_w_store(h, str(p2).encode()) == 0
    lib.orc_w_free(h)
    assert p.read_bytes() == p2.read_bytes()
    idx2 = pado.WeightedVertexCentricPLL()
    idx2.load_index_from_file(str(p))
    qa, qb = G.random_pairs(g.n, 5000, 6)
    assert np.array_equal(idx.query(qa, qb), idx2.query(qa, qb))


def test_import_reference_labels_and_query(pado):
    """Labels made elsewhere (here: the oracle) served by the GPU query kernel."""
    g = G.rmat(11, 8, 15)
    ref = orc.unw_label(g, G.degree_rank(g), 64, 512)
    idx = pado.VertexCentricPLL.from_labels(ref)
    qa, qb = G.random_pairs(g.n, 30000, 9, distinct=False)
    qa[:50] = g.n + 5  # out-of-range ids
    assert np.array_equal(idx.query(qa, qb), orc.unw_query(ref, qa, qb))


def test_query_device_pointers(pado):
    import torch
    g = G.rmat(10, 8, 16)
    idx, lab = gpu_unw(pado, g, G.degree_rank(g), 50, 128)
    qa, qb = G.random_pairs(g.n, 10000, 10)
    a = torch.from_numpy(qa.astype(np.int32)).cuda()
    b = torch.from_numpy(qb.astype(np.int32)).cuda()
    out = torch.empty(10000, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    idx.query_device(a.data_ptr(), b.data_ptr(), out.data_ptr(), 10000, s.cuda_stream)
    s.synchronize()
    assert np.array_equal(out.cpu().numpy(), idx.query(qa, qb))


@pytest.mark.parametrize("weighted", [False, True])
def test_chunked_host_query(pado, weighted):
    """More pairs than one chunk of the host query path (2^21 pairs): the
    chunks alternate between two streams and each chunk's results are read
    back after the next chunk is queued.  Results equal one device launch over
    all pairs and, on a sample, the oracle."""
    import torch
    k = (2 << 21) + 12345
    if weighted:
        g = G.rmat(10, 8, 18, weights=(1, 100))
        idx, lab = gpu_w(pado, g, G.degree_rank(g), 128)
    else:
        g = G.rmat(10, 8, 18)
        idx, lab = gpu_unw(pado, g, G.degree_rank(g), 16, 128)
    qa, qb = G.random_pairs(g.n, k, 11, distinct=False)
    qa[::100003] = g.n + 7  # out-of-range ids in several chunks
    got = idx.query(qa, qb)
    a = torch.from_numpy(qa.view(np.int32)).cuda()
    b = torch.from_numpy(qb.view(np.int32)).cuda()
    out = torch.empty(k, dtype=torch.int16 if weighted else torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    idx.query_device(a.data_ptr(), b.data_ptr(), out.data_ptr(), k, s.cuda_stream)
    s.synchronize()
    assert np.array_equal(got, out.cpu().numpy())
    sel = np.r_[0:2000, (1 << 21) - 1000:(1 << 21) + 1000, k - 2000:k]
    want = (orc.w_query if weighted else orc.unw_query)(lab, qa[sel], qb[sel])
    assert np.array_equal(got[sel], want)


@pytest.mark.parametrize("weighted", [False, True])
def test_export_into_page_locked_buffers(pado, weighted):
    """pado_export writes page-locked destinations from its gather kernel and
    stages pageable ones through device buffers; every mix gives the same
    arrays as an export into pageable memory."""
    import ctypes as C
    import torch
    from parallel_distance_oracle_gb300 import _lib
    if weighted:
        g = G.rmat(11, 8, 19, weights=(1, 100))
        idx, lab = gpu_w(pado, g, G.degree_rank(g), 256)
    else:
        g = G.rmat(11, 8, 19)
        idx, lab = gpu_unw(pado, g, G.degree_rank(g), 40, 256)
    inf = idx.info()
    n, K, tot = inf.n, inf.bp_roots, inf.num_labels
    dt = np.int16 if weighted else np.uint8
    want = [lab.off, lab.hub, lab.dist] + ([lab.bpd, lab.bps] if K else [])
    shapes = [(n + 1, np.uint64), (tot, np.uint32), (tot, dt)] + ([(n * K, np.uint8), (n * K * 2, np.uint64)]
                                                                  if K else [])
    tdt = {np.uint64: torch.int64, np.uint32: torch.int32, np.uint8: torch.uint8, np.int16: torch.int16}
    for pinned in ([True] * len(shapes), [i % 2 == 0 for i in range(len(shapes))],
                   [i % 2 == 1 for i in range(len(shapes))]):
        bufs, views = [], []
        for (cnt, d), pin in zip(shapes, pinned):
            if pin:
                t = torch.zeros(max(cnt, 1), dtype=tdt[d]).pin_memory()
                bufs.append(t)
                views.append(t.numpy().view(d)[:cnt])
            else:
                a = np.zeros(max(cnt, 1), d)
                bufs.append(a)
                views.append(a[:cnt])
        ptrs = [C.c_void_p(b.data_ptr() if isinstance(b, torch.Tensor) else b.ctypes.data) for b in bufs]
        if not K:
            ptrs += [None, None]
        _lib.check(_lib.lib.pado_export(idx._h, *ptrs))
        for got, exp in zip(views, want):
            assert np.array_equal(got, np.asarray(exp).view(got.dtype)[:got.size]), pinned


@pytest.mark.parametrize("n", [1, 2, 5])
def test_tiny_and_edgeless_graphs(pado, n):
    g = G.CSRGraph(n=n, off=np.zeros(n + 1, np.uint64), adj=np.zeros(0, np.uint32))
    rank = np.arange(n, dtype=np.uint32)
    for K in (0, 3):
        idx, lab = gpu_unw(pado, g, rank, K, 4)
        ref = orc.unw_label(g, rank, K, 4)
        assert_same_unw(lab, ref, f"edgeless n={n} K={K}")
        a, b = np.meshgrid(np.arange(n + 1), np.arange(n + 1))
        assert np.array_equal(idx.query(a.ravel(), b.ravel()), orc.unw_query(ref, a.ravel(), b.ravel()))


def test_deterministic_rebuild(pado):
    g = G.rmat(13, 16, 17)
    rank = G.degree_rank(g)
    _, a = gpu_unw(pado, g, rank, 64, 1024)
    _, b = gpu_unw(pado, g, rank, 64, 1024)
    assert_same_unw(a, b, "rebuild")


def test_pool_growth_retry_path_is_exact(pado, monkeypatch):
    """Start the label pool tiny so warps fail to reserve space and are re-run
    after growth; the result must not change."""
    g = G.rmat(11, 8, 18)
    rank = G.degree_rank(g)
    ref = orc.unw_label(g, rank, 16, 256)
    monkeypatch.setenv("PADO_DEBUG_POOL_ENTRIES", "64")
    _, lab = gpu_unw(pado, g, rank, 16, 256)
    assert_same_unw(lab, ref, "tiny pool")
    gw = G.rmat(10, 8, 19, weights=(1, 100))
    rw = G.degree_rank(gw)
    _, lw = gpu_w(pado, gw, rw, 128)
    assert_same_w(lw, orc.w_label(gw, rw, 128), "tiny pool weighted")


def test_device_input_checks(pado):
    """Offsets, adjacency ids and the rank permutation are checked on the
    device after the upload; each bad input fails with PADO_E_ARG."""
    from parallel_distance_oracle_gb300 import _lib
    g = G.path_graph(6)
    bad_rank = np.array([0, 1, 2, 3, 4, 4], np.uint32)
    with pytest.raises(_lib.PadoError, match="permutation"):
        pado.VertexCentricPLL(g, bad_rank, bp_roots=2, batch=4)
    with pytest.raises(_lib.PadoError, match="permutation"):
        pado.VertexCentricPLL(g, np.array([0, 1, 2, 3, 4, 6], np.uint32), bp_roots=2, batch=4)
    b = G.CSRGraph(n=g.n, off=g.off, adj=g.adj.copy())
    b.adj[0] = 99
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.VertexCentricPLL(b, G.degree_rank(g), bp_roots=2, batch=4)
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.VertexCentricPLL(b, None, bp_roots=2, batch=4)
    off = g.off.copy()
    off[3] = off[4] + 1  # decreasing at vertex 3
    with pytest.raises(_lib.PadoError, match="non-decreasing"):
        pado.VertexCentricPLL(G.CSRGraph(n=g.n, off=off, adj=g.adj), None, bp_roots=2, batch=4)
    w = G.rmat(8, 4, 3, weights=(1, 9))
    wb = G.CSRGraph(n=w.n, off=w.off, adj=w.adj.copy(), w=w.w)
    wb.adj[-1] = w.n
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.WeightedVertexCentricPLL(wb, G.degree_rank(w), batch=8)


def test_unsorted_ranked_input_is_sorted_on_the_device(pado):
    """A ranked CSR whose lists are not descending is sorted on the device
    and labels like the sorted one (weights follow their entries)."""
    g = G.rmat(10, 8, 9, weights=(1, 50))
    rk = G.degree_rank(g)
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    ns, nd = rk[src].astype(np.int64), rk[g.adj].astype(np.int64)
    rng = np.random.Generator(np.random.PCG64(2))
    o = np.lexsort((rng.random(len(nd)), ns))  # grouped by source, lists shuffled
    off = np.zeros(g.n + 1, np.uint64)
    np.cumsum(np.bincount(ns, minlength=g.n), out=off[1:])
    shuffled = G.CSRGraph(g.n, off, nd[o].astype(np.uint32), g.w[o])
    a = pado.WeightedVertexCentricPLL(shuffled, None, batch=64).export()
    b = pado.WeightedVertexCentricPLL(g, rk, batch=64)
    b.order_labels(rank=np.arange(g.n, dtype=np.uint32))  # compare keyed by rank on both sides
    b = b.export()
    assert np.array_equal(a.off, b.off) and np.array_equal(a.hub, b.hub) and np.array_equal(a.dist, b.dist)
    ua = pado.VertexCentricPLL(G.CSRGraph(g.n, off, nd[o].astype(np.uint32)), None, bp_roots=8, batch=64).export()
    ub = pado.VertexCentricPLL(g, rk, bp_roots=8, batch=64)
    ub.order_labels(rank=np.arange(g.n, dtype=np.uint32))
    ub = ub.export()
    assert np.array_equal(ua.off, ub.off) and np.array_equal(ua.hub, ub.hub) and np.array_equal(ua.bps, ub.bps)
