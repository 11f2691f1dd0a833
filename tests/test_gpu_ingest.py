"""Device graph ingest (pado_graph_ingest, pado_edge_text_parse,
pado_*_build_edges, pado_build_edge_file) against the oracle's restatement of
the reference's graph preparation (Graph::construct + make_rank with id ties
+ id_transfer, graph.h:95-206) and the reference-made fixtures.  Integer work:
every array must be identical.  Labels built from edges must equal labels
built from the oracle-prepared CSR, and queries by original id must agree."""
import numpy as np
import pytest

from conftest import GOLDEN
from helpers import assert_same_unw, assert_same_w
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

CASES = ["dups_unw", "dups_w", "rmat10_raw", "text_unw", "text_w", "text_unw_nolf"]


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


def same(got, grank, want, wrank, what):
    assert got.n == want.n, what
    assert np.array_equal(grank, wrank), f"{what}: rank"
    assert np.array_equal(np.asarray(got.off, np.uint64), np.asarray(want.off, np.uint64)), f"{what}: offsets"
    assert np.array_equal(got.adj, want.adj), f"{what}: adjacency"
    if want.w is not None:
        assert np.array_equal(got.w, want.w), f"{what}: weights"


@pytest.mark.parametrize("name", CASES)
def test_ingest_matches_reference_golden(pado, name):
    z = np.load(GOLDEN / "ingest_ref.npz")
    if f"{name}_text" in z.files:
        weighted = bool(z[f"{name}_weighted"])
        u, v, w = pado.parse_edge_text(z[f"{name}_text"].tobytes(), weighted)
    else:
        u, v = z[f"{name}_u"], z[f"{name}_v"]
        w = z[f"{name}_w"] if f"{name}_w" in z.files else None
    g, rank = pado.graph_ingest(u, v, w)
    want = G.CSRGraph(int(z[f"{name}_n"]), z[f"{name}_off"], z[f"{name}_adj"],
                      z[f"{name}_wout"] if f"{name}_wout" in z.files else None)
    same(g, rank, want, z[f"{name}_rank"], name)


@pytest.mark.parametrize("dedupe", [False, True])
@pytest.mark.parametrize("weighted", [False, True])
def test_ingest_random_equals_oracle(pado, dedupe, weighted):
    rng = np.random.Generator(np.random.PCG64(11 + 2 * dedupe + weighted))
    for t in range(25):
        n = int(rng.integers(1, 3000))
        m = int(rng.integers(0, 20000))
        u = rng.integers(0, n, m).astype(np.uint32)
        v = rng.integers(0, n, m).astype(np.uint32)
        u[::31] = v[::31]  # self-loops
        u[1::13], v[1::13] = u[::13][: len(u[1::13])], v[::13][: len(u[1::13])]  # repeats
        w = rng.integers(0, 256, m).astype(np.uint8) if weighted else None
        nn = n + int(rng.integers(0, 3))  # isolated top ids when n is given
        got, grank = pado.graph_ingest(u, v, w, n=nn, dedupe=dedupe)
        want, wrank = orc.graph_ingest(u, v, w, n=nn, dedupe=dedupe)
        same(got, grank, want, wrank, f"trial {t} n={nn} m={m}")


@pytest.mark.parametrize("scale,ef", [(14, 16), (16, 8)])
def test_ingest_rmat_raw_samples_many_sort_tiles(pado, scale, ef):
    """Raw R-MAT samples: hundreds of radix-sort tiles, skewed digits.  With
    dedupe the result is the generator's own graph, ranked."""
    n, u, v, w = G.rmat_edges(scale, ef, 3, weights=(1, 100))
    for ww in (None, w):
        got, grank = pado.graph_ingest(u, v, ww, n=n, dedupe=False)
        want, wrank = orc.graph_ingest(u, v, ww, n=n, dedupe=False)
        same(got, grank, want, wrank, f"raw s{scale}")
        got, grank = pado.graph_ingest(u, v, ww, n=n, dedupe=True)
        g = G.csr_from_edges(n, u, v, ww)
        want, wrank = orc.graph_ingest(u, v, ww, n=n, dedupe=True)
        same(got, grank, want, wrank, f"dedupe s{scale}")
        assert np.array_equal(wrank, G.degree_rank(g))


def test_ingest_id_width_edges(pado):
    """Vertex counts at the key-width boundaries (2^k and 2^k + 1)."""
    rng = np.random.Generator(np.random.PCG64(4))
    for n in (1, 2, 3, 255, 256, 257, 65536, 65537, (1 << 20) + 1):
        m = 5000
        u = rng.integers(0, n, m).astype(np.uint32)
        v = rng.integers(0, n, m).astype(np.uint32)
        u[0], v[0] = n - 1, 0
        w = rng.integers(0, 256, m).astype(np.uint8)
        got, grank = pado.graph_ingest(u, v, w, n=n)
        want, wrank = orc.graph_ingest(u, v, w, n=n)
        same(got, grank, want, wrank, f"n={n}")


def test_ingest_empty_and_errors(pado):
    from parallel_distance_oracle_gb300 import _lib
    g, rank = pado.graph_ingest(np.zeros(0, np.uint32), np.zeros(0, np.uint32), n=4)
    assert g.n == 4 and np.array_equal(g.off, np.zeros(5, np.uint64)) and len(g.adj) == 0
    assert np.array_equal(rank, np.arange(4, dtype=np.uint32))
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.graph_ingest(np.array([0, 5], np.uint32), np.array([1, 2], np.uint32), n=5)
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.graph_ingest(np.array([0, 5], np.uint32), np.array([1, 2], np.uint32), n=5, dedupe=True)


def test_text_parse_equals_oracle_including_malformed_lines(pado, monkeypatch):
    rng = np.random.Generator(np.random.PCG64(8))
    junk = [b"", b"   ", b"#c 1 2", b"%c", b"3", b"4 x", b"5 4294967296", b"-1 2", b"x 1 2", b"\r", b" 7 8\r",
            b"+9 +10", b"11\t12 300", b"13 14 abc", b"15 16 99999999999", b"17 18 19 20"]
    lines = []
    for i in range(20000):
        if rng.random() < 0.15:
            lines.append(junk[int(rng.integers(0, len(junk)))])
        else:
            a, b, c = rng.integers(0, 1 << 20), rng.integers(0, 1 << 20), rng.integers(0, 70000)
            lines.append(f"{a} {b} {c}".encode())
    text = b"\n".join(lines)
    for weighted in (False, True):
        want = orc.parse_edge_text(text, weighted)
        got = pado.parse_edge_text(text, weighted)
        for x, y in zip(got, want):
            assert (x is None and y is None) or np.array_equal(x, y)
        # pieces far smaller than the text: lines meet piece ends
        monkeypatch.setenv("PADO_DEBUG_TEXT_PIECE", "4099")
        got = pado.parse_edge_text(text, weighted)
        monkeypatch.delenv("PADO_DEBUG_TEXT_PIECE")
        for x, y in zip(got, want):
            assert (x is None and y is None) or np.array_equal(x, y)
    assert all(len(a) == 0 for a in pado.parse_edge_text(b"", False)[:2])
    assert len(pado.parse_edge_text(b"\n\n# only comments\n", False)[0]) == 0


def labels_of(idx, K):
    lab = idx.export()
    return orc.UnwLabels(lab.n, K, lab.off, lab.hub, lab.dist,
                         lab.bpd if K else np.zeros(0, np.uint8), lab.bps if K else np.zeros(0, np.uint64))


def test_build_edges_equals_build_from_prepared_csr(pado):
    n, u, v, _ = G.rmat_edges(12, 8, 21)
    K, B = 16, 128
    idx = pado.VertexCentricPLL.from_edges(u, v, n=n, dedupe=True, bp_roots=K, batch=B)
    g = G.csr_from_edges(n, u, v)
    rank = G.degree_rank(g)
    ref = pado.VertexCentricPLL(g, rank, bp_roots=K, batch=B)
    assert_same_unw(labels_of(idx, K), labels_of(ref, K), "rmat12 from edges")
    qa, qb = G.random_pairs(n, 5000, 3, distinct=False)
    assert np.array_equal(idx.query(qa, qb), ref.query(qa, qb))
    # without dedupe the reference's Graph semantics: repeats and self-loops
    # kept, n = max id + 1; compared with the oracle labeling the oracle-
    # prepared ranked graph, row v of the edges-built index being row rank[v]
    idx2 = pado.VertexCentricPLL.from_edges(u, v, bp_roots=K, batch=B)
    g2, r2 = orc.graph_ingest(u, v)
    lab = orc.unw_label(g2, np.arange(g2.n, dtype=np.uint32), K, B)
    got = labels_of(idx2, K)
    assert got.n == g2.n
    cnt = np.diff(lab.off.astype(np.int64))
    rows = np.repeat(np.asarray(lab.off[:-1], np.int64)[r2], cnt[r2]) + (
        np.arange(int(cnt[r2].sum())) - np.repeat(np.cumsum(cnt[r2]) - cnt[r2], cnt[r2]))
    assert np.array_equal(np.diff(got.off.astype(np.int64)), cnt[r2])
    assert np.array_equal(got.hub, lab.hub[rows]) and np.array_equal(got.dist, lab.dist[rows])
    bpd = np.asarray(lab.bpd).reshape(g2.n, K)[r2]
    bps = np.asarray(lab.bps).reshape(g2.n, 2 * K)[r2]
    assert np.array_equal(np.asarray(got.bpd).reshape(g2.n, K), bpd)
    assert np.array_equal(np.asarray(got.bps).reshape(g2.n, 2 * K), bps)
    qa = (qa % g2.n).astype(np.uint32)
    qb = (qb % g2.n).astype(np.uint32)
    assert np.array_equal(idx2.query(qa, qb), orc.unw_query(lab, r2[qa], r2[qb]))


def test_weighted_build_edges_equals_build_from_prepared_csr(pado):
    n, u, v, w = G.rmat_edges(11, 8, 22, weights=(1, 100))
    idx = pado.WeightedVertexCentricPLL.from_edges(u, v, w, n=n, dedupe=True, batch=128)
    g = G.csr_from_edges(n, u, v, w)
    ref = pado.WeightedVertexCentricPLL(g, G.degree_rank(g), batch=128)
    a, b = idx.export(), ref.export()
    assert_same_w(orc.WLabels(a.n, a.off, a.hub, a.dist), orc.WLabels(b.n, b.off, b.hub, b.dist), "weighted")
    qa, qb = G.random_pairs(n, 5000, 4, distinct=False)
    assert np.array_equal(idx.query(qa, qb), ref.query(qa, qb))


@pytest.mark.parametrize("weighted", [False, True])
def test_build_edge_file_equals_build_from_arrays(pado, tmp_path, monkeypatch, weighted):
    n, u, v, w = G.rmat_edges(11, 8, 23, weights=(1, 100))
    rows = [f"{a}\t{b}\t{c}" if weighted else f"{a} {b}" for a, b, c in zip(u, v, w)]
    path = tmp_path / "edges.txt"
    path.write_text("# header\n" + "\n".join(rows) + "\n")
    monkeypatch.setenv("PADO_DEBUG_TEXT_PIECE", "65536")  # several read pieces
    if weighted:
        idx = pado.WeightedVertexCentricPLL.from_edge_file(path, dedupe=True, batch=64)
        ref = pado.WeightedVertexCentricPLL.from_edges(u, v, w, dedupe=True, batch=64)
    else:
        idx = pado.VertexCentricPLL.from_edge_file(path, dedupe=True, bp_roots=8, batch=64)
        ref = pado.VertexCentricPLL.from_edges(u, v, dedupe=True, bp_roots=8, batch=64)
    a, b = idx.export(), ref.export()
    assert a.n == b.n
    assert np.array_equal(a.off, b.off) and np.array_equal(a.hub, b.hub) and np.array_equal(a.dist, b.dist)
    qa, qb = G.random_pairs(a.n, 3000, 5, distinct=False)
    assert np.array_equal(idx.query(qa, qb), ref.query(qa, qb))


def test_build_edge_file_missing_is_io_error(pado, tmp_path):
    from parallel_distance_oracle_gb300 import _lib
    with pytest.raises(_lib.PadoError, match="cannot open"):
        pado.VertexCentricPLL.from_edge_file(tmp_path / "absent.txt")


def test_ingest_device_pointers_equal_host_call(pado):
    """pado_graph_ingest_device on torch device tensors, on a caller stream."""
    import ctypes as C

    import torch
    from parallel_distance_oracle_gb300 import _lib
    n, u, v, w = G.rmat_edges(13, 8, 6, weights=(1, 100))
    u, v = u.astype(np.uint32), v.astype(np.uint32)
    m = len(u)
    want, wrank = pado.graph_ingest(u, v, w, n=n)
    du = torch.from_numpy(u.view(np.int32)).cuda()
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    dw = torch.from_numpy(w).cuda()
    off = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    adj = torch.zeros(2 * m, dtype=torch.int32, device="cuda")
    wo = torch.zeros(2 * m, dtype=torch.uint8, device="cuda")
    rank = torch.zeros(n, dtype=torch.int32, device="cuda")
    ent = C.c_uint64()
    s = torch.cuda.Stream()
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _lib.check(_lib.lib.pado_graph_ingest_device(m, P(du), P(dv), P(dw), n, 0, P(off), P(adj), P(wo), P(rank),
                                                 C.byref(ent), C.c_void_p(s.cuda_stream)))
    assert ent.value == len(want.adj)
    assert np.array_equal(off.cpu().numpy().view(np.uint64), want.off)
    assert np.array_equal(adj.cpu().numpy().view(np.uint32), want.adj)
    assert np.array_equal(wo.cpu().numpy(), want.w)
    assert np.array_equal(rank.cpu().numpy().view(np.uint32), wrank)


def test_scratch_cache_keeps_results(pado):
    """With scratch kept between calls, repeated ingests give the same CSR."""
    from parallel_distance_oracle_gb300 import _lib
    n, u, v, _ = G.rmat_edges(12, 8, 7)
    want, wrank = orc.graph_ingest(u, v, n=n)
    _lib.check(_lib.lib.pado_set_scratch_cache(1 << 30))
    try:
        for _ in range(3):
            got, grank = pado.graph_ingest(u, v, n=n)
            same(got, grank, want, wrank, "cached scratch")
    finally:
        _lib.check(_lib.lib.pado_set_scratch_cache(0))
