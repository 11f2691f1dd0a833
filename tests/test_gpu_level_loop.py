"""The two drivers of the labeling loops give the same labels.

The product path runs every batch and level (round) of a build inside one
persistent cooperative launch; PADO_LEVEL_LOOP=host runs the same device code
as one launch per phase, driven by the host (the form used for ncu captures
of single levels).  The persistent weighted loop marks the next round's tails
inside the pull and merges the end-of-batch filter and commit, where the host
loop keeps separate mark, filter and commit launches, so equal labels from
both, and equal to the oracle, check those merged phases."""
import numpy as np
import pytest

from helpers import assert_same_unw, assert_same_w
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado
    return pado


@pytest.mark.parametrize("scale,ef,seed,B", [(11, 8, 41, 64), (12, 8, 42, 128), (13, 8, 43, 512)])
def test_weighted_host_loop_equals_persistent_loop(pado, monkeypatch, scale, ef, seed, B):
    g = G.rmat(scale, ef, seed, weights=(1, 100))
    rank = G.degree_rank(g)
    monkeypatch.delenv("PADO_LEVEL_LOOP", raising=False)
    a = pado.WeightedVertexCentricPLL(g, rank, batch=B).export()
    monkeypatch.setenv("PADO_LEVEL_LOOP", "host")
    b = pado.WeightedVertexCentricPLL(g, rank, batch=B).export()
    assert np.array_equal(a.off, b.off) and np.array_equal(a.hub, b.hub) and np.array_equal(a.dist, b.dist)
    assert_same_w(a, orc.w_label(g, rank, B), "persistent loop")


@pytest.mark.parametrize("scale,ef,seed,K,B", [(11, 8, 44, 16, 64), (12, 16, 45, 64, 256)])
def test_unweighted_host_loop_equals_persistent_loop(pado, monkeypatch, scale, ef, seed, K, B):
    g = G.rmat(scale, ef, seed)
    rank = G.degree_rank(g)
    monkeypatch.delenv("PADO_LEVEL_LOOP", raising=False)
    a = pado.VertexCentricPLL(g, rank, bp_roots=K, batch=B).export()
    monkeypatch.setenv("PADO_LEVEL_LOOP", "host")
    b = pado.VertexCentricPLL(g, rank, bp_roots=K, batch=B).export()
    assert_same_unw(a, b, "host loop")
    assert_same_unw(a, orc.unw_label(g, rank, K, B), "persistent loop")


def test_weighted_tiny_round_log_with_host_loop(pado, monkeypatch):
    """The host loop's own log-growth re-run, from tiny initial capacities."""
    g = G.rmat(10, 8, 46, weights=(1, 100))
    rank = G.degree_rank(g)
    monkeypatch.setenv("PADO_DEBUG_POOL_ENTRIES", "64")
    monkeypatch.setenv("PADO_LEVEL_LOOP", "host")
    lab = pado.WeightedVertexCentricPLL(g, rank, batch=128).export()
    assert_same_w(lab, orc.w_label(g, rank, 128), "tiny pool, host loop")
