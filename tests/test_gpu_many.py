"""Many graphs labeled together (pado_unw_build_many): every graph's labels
and BP rows must be exactly those of labeling it alone -- against the oracle
for each graph and against the one-graph GPU build -- and its queries must
equal the oracle's.  The mix covers what the batched loop has to keep apart:
graphs of very different sizes (so they finish batches at different steps),
graphs with fewer vertices than BP roots, a graph whose first batches are all
BP vertices, edgeless and one-vertex graphs, and a pool small enough that the
loop stops for growth in the middle of a step."""
import numpy as np
import pytest

from helpers import assert_same_unw
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


def as_labels(idx, K):
    lab = idx.export()
    return orc.UnwLabels(lab.n, K, lab.off, lab.hub, lab.dist,
                         lab.bpd if K else np.zeros(0, np.uint8), lab.bps if K else np.zeros(0, np.uint64))


def mixed_graphs(count, seed, n_lo=200, n_hi=3000):
    rng = np.random.Generator(np.random.PCG64(seed))
    gs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        if i % 2 == 0:
            gs.append(G.erdos_renyi(n, 6, seed * 1000 + i))
        else:
            gs.append(G.grid_with_shortcuts(n, 0.02, seed * 1000 + i))
    return gs


def edgeless(n):
    return G.CSRGraph(n=n, off=np.zeros(n + 1, np.uint64), adj=np.zeros(0, np.uint32))


@pytest.mark.parametrize("K,B", [(16, 64), (0, 128), (50, 256)])
def test_many_equals_oracle_per_graph(pado, K, B):
    gs = mixed_graphs(12, 3 + K) + [edgeless(1), edgeless(5), G.path_graph(40), G.rmat(9, 8, 5)]
    ranks = [G.degree_rank(g) for g in gs]
    idxs = pado.build_many(gs, ranks, bp_roots=K, batch=B)
    assert len(idxs) == len(gs)
    for i, (g, rk, idx) in enumerate(zip(gs, ranks, idxs)):
        ref = orc.unw_label(g, rk, K, B)
        assert_same_unw(as_labels(idx, K), ref, f"graph {i} (n={g.n})")
        qa, qb = G.random_pairs(max(g.n, 2), 3000, 11 + i, distinct=False)
        assert np.array_equal(idx.query(qa, qb), orc.unw_query(ref, qa, qb)), f"graph {i} queries"


def test_many_equals_one_at_a_time(pado):
    """Same labels as the one-graph GPU build, graph by graph, at a size the
    oracle would be slow for."""
    gs = mixed_graphs(6, 21, 5000, 20000) + [G.rmat(13, 8, 22)]
    ranks = [G.degree_rank(g) for g in gs]
    idxs = pado.build_many(gs, ranks, bp_roots=64, batch=512)
    for i, (g, rk, idx) in enumerate(zip(gs, ranks, idxs)):
        alone = pado.VertexCentricPLL(g, rk, bp_roots=64, batch=512)
        assert_same_unw(as_labels(idx, 64), as_labels(alone, 64), f"graph {i} (n={g.n})")


def test_many_ranked_input_and_single_graph(pado):
    """rank None means the ids are already ranks; one graph alone also works."""
    g = G.grid_with_shortcuts(900, 0.02, 7)
    rk = G.degree_rank(g)
    # relabel to rank ids, as Graph::id_transfer does
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    gr = G.csr_from_edges(g.n, rk[src].astype(np.int64), rk[g.adj.astype(np.int64)].astype(np.int64))
    (idx,) = pado.build_many([gr], None, bp_roots=8, batch=64)
    ref = orc.unw_label(gr, np.arange(g.n, dtype=np.uint32), 8, 64)
    assert_same_unw(as_labels(idx, 8), ref, "ranked")


def test_many_pool_growth_mid_step_is_exact(pado, monkeypatch):
    gs = mixed_graphs(8, 31, 300, 2500)
    ranks = [G.degree_rank(g) for g in gs]
    monkeypatch.setenv("PADO_DEBUG_POOL_ENTRIES", "64")
    idxs = pado.build_many(gs, ranks, bp_roots=16, batch=128)
    for i, (g, rk, idx) in enumerate(zip(gs, ranks, idxs)):
        assert_same_unw(as_labels(idx, 16), orc.unw_label(g, rk, 16, 128), f"graph {i} (n={g.n})")


def test_many_rejects_bad_input_and_returns_no_handles(pado):
    from parallel_distance_oracle_gb300 import _lib
    g = G.path_graph(10)
    bad = G.CSRGraph(n=3, off=np.array([0, 1, 2, 3], np.uint64), adj=np.array([1, 7, 0], np.uint32))
    with pytest.raises(_lib.PadoError, match="out of range"):
        pado.build_many([g, bad], None, bp_roots=2, batch=8)
    with pytest.raises(_lib.PadoError, match="batch"):
        pado.build_many([g], None, bp_roots=2, batch=4096)


def test_tune_batch_picks_a_candidate(pado):
    gs = mixed_graphs(10, 41, 500, 4000)
    ranks = [G.degree_rank(g) for g in gs]
    best, ms = pado.tune_batch(gs, ranks, bp_roots=16, candidates=(64, 256, 1024), sample=4)
    assert best in (64, 256, 1024)
    assert set(ms) == {64, 256, 1024} and all(t > 0 for t in ms.values())
    assert ms[best] == min(ms.values())
