import numpy as np

from parallel_distance_oracle_gb300 import graphs as G


def _check_simple(g):
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    dst = g.adj.astype(np.int64)
    assert not np.any(src == dst), "self-loop"
    key = src * g.n + dst
    assert len(np.unique(key)) == len(key), "duplicate"
    rkey = dst * g.n + src
    assert np.array_equal(np.sort(key), np.sort(rkey)), "not symmetric"


def test_rmat_deterministic_and_simple():
    a, b = G.rmat(10, 8, 5), G.rmat(10, 8, 5)
    assert np.array_equal(a.adj, b.adj) and np.array_equal(a.off, b.off)
    assert a.n == 1024
    _check_simple(a)
    c = G.rmat(10, 8, 6)
    assert not np.array_equal(a.adj, c.adj) or not np.array_equal(a.off, c.off)


def test_weighted_rmat_symmetric_weights():
    g = G.rmat(9, 8, 3, weights=(1, 100))
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    fw = {(int(u), int(v)): int(w) for u, v, w in zip(src, g.adj, g.w)}
    for (u, v), w in list(fw.items())[:500]:
        assert fw[(v, u)] == w
    assert g.w.min() >= 1 and g.w.max() <= 100


def test_er_and_grid():
    _check_simple(G.erdos_renyi(1000, 6, 1))
    g = G.grid_with_shortcuts(1000, 0.02, 2)
    _check_simple(g)
    assert g.m_directed >= 2 * (2 * 1000 - 2 * 32)


def test_degree_rank_is_permutation_desc_degree_tie_by_id():
    g = G.rmat(9, 8, 1)
    r = G.degree_rank(g)
    assert np.array_equal(np.sort(r), np.arange(g.n))
    order = np.argsort(r)
    deg = g.degrees()[order]
    assert np.all(deg[:-1] >= deg[1:])
    for i in range(g.n - 1):
        if deg[i] == deg[i + 1]:
            assert order[i] < order[i + 1]


def test_random_pairs_distinct():
    a, b = G.random_pairs(100, 5000, 3)
    assert np.all(a != b) and a.max() < 100


def test_keep_duplicates_matches_reference_graph_construct():
    g = G.csr_keep_duplicates(4, [0, 1, 0, 2], [1, 2, 1, 2])
    # vertex 2's list: 1 (edge 1), then 2, 2 (self-loop pushed twice)
    assert list(g.adj[g.off[2]:g.off[3]]) == [1, 2, 2]
    assert list(g.adj[g.off[0]:g.off[1]]) == [1, 1]
