"""The CPU oracle is pinned against golden vectors produced by the reference
itself (tests/golden/make_golden.py), and against BFS / Dijkstra."""
import numpy as np
import pytest

from conftest import golden_cases
from helpers import assert_same_unw, assert_same_w, golden_unw_labels, golden_w_labels, load_golden
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G


@pytest.mark.parametrize("path", golden_cases("unw"), ids=lambda p: p.stem)
def test_oracle_unweighted_matches_reference_golden(path):
    z, g = load_golden(path)
    lab = orc.unw_label(g, z["rank"], int(z["K"]), int(z["B"]))
    assert_same_unw(lab, golden_unw_labels(z), path.stem)
    q = orc.unw_query(lab, z["qa"], z["qb"])
    assert np.array_equal(q, z["qd"])


@pytest.mark.parametrize("path", golden_cases("w"), ids=lambda p: p.stem)
def test_oracle_weighted_matches_reference_golden(path):
    z, g = load_golden(path)
    lab = orc.w_label(g, z["rank"], int(z["B"]))
    assert_same_w(lab, golden_w_labels(z), path.stem)
    q = orc.w_query(lab, z["qa"], z["qb"])
    assert np.array_equal(q, z["qd"])


@pytest.mark.parametrize("path", golden_cases("w"), ids=lambda p: p.stem)
def test_oracle_level_synchronous_weighted_schedule_matches_golden(path):
    # mode 5 = the schedule the GPU runs: snapshot check (2) + snapshot filter
    z, g = load_golden(path)
    lab = orc.w_label(g, z["rank"], int(z["B"]), mode=5)
    assert_same_w(lab, golden_w_labels(z), path.stem)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_queries_equal_bfs(seed):
    g = G.rmat(10, 8, seed)
    lab = orc.unw_label(g, G.degree_rank(g), 50, 64)
    a, b = G.random_pairs(g.n, 300, seed + 100)
    q = orc.unw_query(lab, a, b)
    for i in range(0, 300, 3):
        assert q[i] == orc.bfs(g, int(a[i]))[b[i]]


@pytest.mark.parametrize("seed", [4, 5])
def test_oracle_weighted_queries_equal_dijkstra(seed):
    g = G.rmat(10, 8, seed, weights=(1, 100))
    lab = orc.w_label(g, G.degree_rank(g), 128)
    a, b = G.random_pairs(g.n, 200, seed + 100)
    q = orc.w_query(lab, a, b)
    for i in range(0, 200, 2):
        assert q[i] == orc.dijkstra(g, int(a[i]))[b[i]]


def test_oracle_c1_config_against_bfs():
    # R-MAT s14 / ef 8 / K=50 / B=1024, sampled against BFS
    g = G.rmat(14, 8, 1)
    lab = orc.unw_label(g, G.degree_rank(g), 50, 1024)
    a, b = G.random_pairs(g.n, 2000, 11)
    q = orc.unw_query(lab, a, b)
    for i in range(0, 2000, 40):
        assert q[i] == orc.bfs(g, int(a[i]))[b[i]]


def test_reference_live_if_built():
    """Where the reference was compiled here, check the oracle against it on
    fresh seeds too (skipped on hosts without the reference build)."""
    if not orc.ref_available(50):
        pytest.skip("reference driver not built on this host")
    for seed in (31, 32):
        g = G.rmat(11, 8, seed)
        rk = G.degree_rank(g)
        assert orc.same_unw(orc.unw_label(g, rk, 50, 256), orc.ref_unw_label(g, rk, 50, 256, mode=1, threads=4))
        gw = G.rmat(10, 8, seed, weights=(1, 100))
        rk = G.degree_rank(gw)
        assert orc.same_w(orc.w_label(gw, rk, 128), orc.ref_w_label(gw, rk, 128, mode=1, threads=4))
