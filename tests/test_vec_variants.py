"""The reference's AVX-512 labelers (pado.cpp's `-v 1` modes: pado.cpp:239-261
VertexCentricPLLVec<1024> / ParaVertexCentricPLLVec<1024>, :297-341
WeightedVertexCentricPLLVec<512> / WeightedParaVertexCentricPLLVec<512>)
against the scalar classes the GPU labelers are pinned to.  The drop-in header
maps the `*Vec` class names onto the same GPU labelers; these tests record what
that mapping gives a `-v 1` user.

* Weighted: the AVX-512 classes (sequential and OpenMP) produce exactly the
  scalar classes' canonical labels.
* Unweighted: on some graphs the AVX-512 classes leave out the distance-1 label
  of a degree-1 vertex to its only neighbour, and their own query then answers
  unreachable for that adjacent pair.  Every label they lack is of that kind,
  they add none, and wherever they differ the scalar labels (and so the GPU's)
  answer every pair as BFS does.  Elsewhere the labels are identical.

Needs an x86 CPU with AVX-512 (the reference's own target); skipped elsewhere."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import assert_same_w, golden_unw_labels, golden_w_labels, load_golden
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.skipif(not orc.refvec_available(), reason="no AVX-512 CPU / reference tree on this host")


@pytest.mark.parametrize("case", ["w_rmat9_w100_b64", "w_rmat10_w7_b128", "w_ref_weighted_edgelist_b512",
                                  "w_grid400_w3_b32"])
@pytest.mark.parametrize("mode", [0, 1])
def test_weighted_vec_equals_scalar_golden(case, mode):
    z, g = load_golden(GOLDEN / f"{case}.npz")
    B = int(z["B"])
    if B < 64:
        pytest.skip("the AVX-512 driver is instantiated for batches of 64 and more")
    v = orc.refvec_label(g, z["rank"], B, True, mode, threads=4)
    assert_same_w(v, golden_w_labels(z), case)


@pytest.mark.parametrize("scale,seed,B", [(11, 5, 512), (12, 6, 512), (12, 7, 1024)])
def test_weighted_vec_equals_scalar_rmat(scale, seed, B):
    g = G.rmat(scale, 8, seed, weights=(1, 100))
    rank = G.degree_rank(g)
    ref = orc.ref_w_label(g, rank, B)
    for mode in (0, 1):
        assert_same_w(orc.refvec_label(g, rank, B, True, mode, threads=4), ref, f"mode {mode}")


@pytest.mark.parametrize("case", ["unw_rmat9_k50_b64", "unw_ref_edgelist_k50"])
@pytest.mark.parametrize("mode", [0, 1])
def test_unweighted_vec_equals_scalar_golden(case, mode):
    z, g = load_golden(GOLDEN / f"{case}.npz")
    v = orc.refvec_label(g, z["rank"], int(z["B"]), False, mode, threads=4)
    assert orc.same_unw(v, golden_unw_labels(z))


@pytest.mark.parametrize("scale,seed,B", [(11, 3, 256), (12, 4, 1024), (11, 6, 1024), (12, 8, 512)])
def test_unweighted_vec_drops_degree1_labels(scale, seed, B):
    g = G.rmat(scale, 8, seed)
    rank = G.degree_rank(g)
    ref = orc.ref_unw_label(g, rank, 50, B)
    deg = np.diff(g.off.astype(np.int64))
    r2i = np.argsort(rank)
    for mode in (0, 1):
        v = orc.refvec_label(g, rank, B, False, mode, threads=4)
        assert np.array_equal(v.bpd, ref.bpd) and np.array_equal(v.bps, ref.bps)
        missing = 0
        for x in range(g.n):
            a = set(zip(ref.hub[ref.off[x]:ref.off[x + 1]].tolist(), ref.dist[ref.off[x]:ref.off[x + 1]].tolist()))
            b = set(zip(v.hub[v.off[x]:v.off[x + 1]].tolist(), v.dist[v.off[x]:v.off[x + 1]].tolist()))
            assert b <= a, f"vertex {x}: the AVX-512 class adds labels"
            for hub, d in a - b:
                # the dropped label: degree-1 vertex, distance 1, hub = its only neighbour
                assert deg[x] == 1 and d == 1 and r2i[hub] == g.adj[g.off[x]]
                nb = np.array([r2i[hub]], np.uint32)
                assert orc.unw_query(v, np.array([x], np.uint32), nb)[0] == 255
                assert orc.unw_query(ref, np.array([x], np.uint32), nb)[0] == 1
                missing += 1
        if missing:
            # the scalar labels answer every pair from the affected vertices as BFS does
            xs = [x for x in range(g.n) if v.off[x + 1] - v.off[x] != ref.off[x + 1] - ref.off[x]]
            for x in xs[:5]:
                allb = np.arange(g.n, dtype=np.uint32)
                assert np.array_equal(orc.unw_query(ref, np.full(g.n, x, np.uint32), allb), orc.bfs(g, x))
