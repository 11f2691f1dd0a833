"""Graph preparation in the oracle (orc_graph_ingest, orc_edge_text_parse) is
pinned to the reference's own Graph code: the committed fixtures made by
tests/golden/make_ingest_golden.py, and -- where the reference tree and the
compiled reference driver are present -- the reference run directly on random
edge lists and on the reference's own fixture files.  Dedupe is pinned to the
benchmark generator's cleaning (graphs.csr_from_edges)."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import build_oracle, orc
from parallel_distance_oracle_gb300 import graphs as G

REF_TOOLS = build_oracle._reference_dir() / "tools"  # the reference's fixture files
CASES = ["dups_unw", "dups_w", "rmat10_raw", "text_unw", "text_w", "text_unw_nolf"]


def golden():
    return np.load(GOLDEN / "ingest_ref.npz")


def same_csr(g, rank, z, name):
    assert g.n == int(z[f"{name}_n"]), name
    assert np.array_equal(rank, z[f"{name}_rank"]), f"{name}: rank"
    assert np.array_equal(np.asarray(g.off, np.uint64), z[f"{name}_off"]), f"{name}: offsets"
    assert np.array_equal(g.adj, z[f"{name}_adj"]), f"{name}: adjacency"
    if f"{name}_wout" in z.files:
        assert np.array_equal(g.w, z[f"{name}_wout"]), f"{name}: weights"


def ranked_reference_of(g):
    """Expected ranked CSR of a deduplicated generator graph: degree rank with
    ascending-id ties, lists descending."""
    rank = G.degree_rank(g)
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    ns, nd = rank[src].astype(np.int64), rank[g.adj].astype(np.int64)
    o = np.lexsort((-nd, ns))
    off = np.zeros(g.n + 1, np.uint64)
    np.cumsum(np.bincount(ns, minlength=g.n), out=off[1:])
    return G.CSRGraph(g.n, off, nd[o].astype(np.uint32), None if g.w is None else g.w[o]), rank


@pytest.mark.parametrize("name", CASES)
def test_oracle_ingest_matches_reference_golden(name):
    z = golden()
    if f"{name}_text" in z.files:
        weighted = bool(z[f"{name}_weighted"])
        u, v, w = orc.parse_edge_text(z[f"{name}_text"].tobytes(), weighted)
    else:
        u, v = z[f"{name}_u"], z[f"{name}_v"]
        w = z[f"{name}_w"] if f"{name}_w" in z.files else None
    g, rank = orc.graph_ingest(u, v, w)
    same_csr(g, rank, z, name)


def test_oracle_dedupe_matches_generator_cleaning():
    rng = np.random.Generator(np.random.PCG64(5))
    for t in range(40):
        n = int(rng.integers(2, 90))
        m = int(rng.integers(1, 400))
        u, v = rng.integers(0, n, m), rng.integers(0, n, m)
        w = rng.integers(1, 101, m).astype(np.uint8)
        for ww in (None, w):
            want, wrank = ranked_reference_of(G.csr_from_edges(n, u, v, ww))
            got, rank = orc.graph_ingest(u, v, ww, n=n, dedupe=True)
            assert np.array_equal(rank, wrank), t
            assert np.array_equal(got.off, want.off) and np.array_equal(got.adj, want.adj), t
            if ww is not None:
                assert np.array_equal(got.w, want.w), t


def test_oracle_text_rules_on_malformed_lines():
    text = (b"1 2\n\n   \n#x\n%y\n3\n4 x\n5 4294967296\n4294967295 1\n+6 +7\n8\t9 300\n"
            b"10 11 abc\n12 13 99999999999\n-1 2\n 14 15\r\n16 17")
    u, v, _ = orc.parse_edge_text(text, False)
    assert u.tolist() == [1, 4294967295, 6, 8, 10, 12, 14, 16]
    assert v.tolist() == [2, 1, 7, 9, 11, 13, 15, 17]
    u, v, w = orc.parse_edge_text(text, True)
    assert w.tolist() == [0, 0, 0, 300 % 256, 0, 255, 0, 0]


needs_ref = pytest.mark.skipif(not (REF_TOOLS.exists() and orc.ref_available(50)),
                               reason="reference tree or compiled reference driver absent")


@needs_ref
def test_oracle_ingest_matches_reference_on_random_edge_lists():
    rng = np.random.Generator(np.random.PCG64(9))
    for t in range(40):
        n = int(rng.integers(1, 70))
        m = int(rng.integers(1, 300))
        u = rng.integers(0, n, m).astype(np.uint32)
        v = rng.integers(0, n, m).astype(np.uint32)
        w = rng.integers(0, 256, m).astype(np.uint8)
        for ww in (None, w):
            want, wrank = orc.ref_graph_edges(u, v, ww)
            got, rank = orc.graph_ingest(u, v, ww)
            assert got.n == want.n and np.array_equal(rank, wrank), t
            assert np.array_equal(got.off, want.off) and np.array_equal(got.adj, want.adj), t
            if ww is not None:
                assert np.array_equal(got.w, want.w), t


@needs_ref
@pytest.mark.parametrize("name,weighted", [("edgelist.in", False), ("triangle.in", False),
                                           ("rectangle.in", False), ("deleted_graph.in", False),
                                           ("weighted_edgelist.in", True), ("1_w_edgelist.in", True),
                                           ("7_w_edgelist.in", True)])
def test_oracle_text_matches_reference_reader_on_its_fixtures(name, weighted):
    path = REF_TOOLS / name
    want, wrank = orc.ref_graph_file(path, weighted)
    u, v, w = orc.parse_edge_text(path.read_bytes(), weighted)
    got, rank = orc.graph_ingest(u, v, w)
    assert got.n == want.n and np.array_equal(rank, wrank)
    assert np.array_equal(got.off, want.off) and np.array_equal(got.adj, want.adj)
    if weighted:
        assert np.array_equal(got.w, want.w)
