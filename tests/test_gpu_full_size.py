"""Full-size parity on the three headline graphs (R-MAT s14 / K=50, R-MAT s20
ef16 / K=64 / B=1024, weighted R-MAT s18 / B=512), against digests the
compiled reference made (tests/golden/make_golden.py --digests and
--digests-extra):

* labels: the GPU labels hash to the same SHA-256 as the reference's own
  OpenMP labeler's canonical labels (offsets, hubs, distances and, unweighted,
  the BP rows), so the label sets are bit-identical;
* queries: the GPU's answers to the workload's own query pairs (100k, 10M and
  1M uniform pairs, seeds 11 / 12 / 13) hash to the SHA-256 of the reference's
  query_distance answers over its own labels (pado_unw_unv_unp.h:1312-1445,
  pado_weighted_unv_unp.h:1782-1900), and 2,000 pairs under 20 of those
  sources equal a plain BFS / Dijkstra from the source, except where the
  reference's own query skips a bit-parallel root (see below);
* index file: pado_store writes the same bytes as the reference's
  store_index_to_file on the same labeling (digest of the whole file)."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

CASES = json.loads((GOLDEN / "full_size_digests.json").read_text())


def digest(kind, off, hub, dist, bpd=None, bps=None):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(hub, np.uint32).tobytes())
    h.update(np.ascontiguousarray(dist, np.uint8 if kind == "unw" else np.int16).tobytes())
    if bpd is not None and len(bpd):
        h.update(np.ascontiguousarray(bpd, np.uint8).tobytes())
        h.update(np.ascontiguousarray(bps, np.uint64).tobytes())
    return h.hexdigest()


def file_digest(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 24), b""):
            h.update(chunk)
    return h.hexdigest()


@pytest.fixture(scope="module", params=sorted(CASES))
def built(request, cuda_ok):
    """The case's graph labeled on the GPU once for all checks below."""
    from parallel_distance_oracle_gb300 import pado
    name = request.param
    c = CASES[name]
    w = (1, 100) if c["kind"] == "w" else None
    g = G.rmat(c["scale"], c["ef"], c["seed"], weights=w)
    rank = G.degree_rank(g)
    if c["kind"] == "unw":
        idx = pado.VertexCentricPLL(g, rank, bp_roots=c["K"], batch=c["B"])
    else:
        idx = pado.WeightedVertexCentricPLL(g, rank, batch=c["B"])
    yield name, c, g, idx
    idx.close()


def test_full_size_labels_match_reference_digest(built):
    name, c, g, idx = built
    lab = idx.export()
    if c["kind"] == "unw":
        got = digest("unw", lab.off, lab.hub, lab.dist, lab.bpd, lab.bps)
    else:
        got = digest("w", lab.off, lab.hub, lab.dist)
    assert int(idx.info().num_labels) == c["labels"]
    assert got == c["sha256"]


def test_full_size_queries_match_reference_and_bfs(built):
    name, c, g, idx = built
    q = c["queries"]
    qa, qb = G.random_pairs(g.n, q["count"], q["seed"])
    ans = idx.query(qa, qb)
    assert ans.dtype == (np.uint8 if c["kind"] == "unw" else np.int16)
    assert hashlib.sha256(np.ascontiguousarray(ans).tobytes()).hexdigest() == q["sha256"]
    # 20 sources (the first pair endpoints), 100 targets each, against BFS /
    # Dijkstra.  One documented exception, the reference's own: its query
    # compares `int td - 2` with an unsigned bound (pado_unw_unv_unp.h:1345),
    # so a bit-parallel root whose two BP distances sum to less than 2 (the
    # root itself and one of its chosen neighbours) is skipped, and such an
    # adjacent pair can come out longer than 1.  The GPU reproduces the
    # reference's answer there (the digest above covers it).
    K = int(c["K"])
    bpd = idx.export().bpd.reshape(g.n, K) if K else None
    rng = np.random.Generator(np.random.PCG64(q["seed"] + 1000))
    for s in qa[:20]:
        tg = rng.integers(0, g.n, 100).astype(np.uint32)
        got = idx.query(np.full(100, s, np.uint32), tg).astype(np.int64)
        truth = (orc.bfs(g, int(s)) if c["kind"] == "unw" else orc.dijkstra(g, int(s)))[tg].astype(np.int64)
        for i in np.nonzero(got != truth)[0]:
            assert K and got[i] > truth[i], f"{name}: source {s} target {tg[i]}"
            sums = bpd[s].astype(np.int64) + bpd[tg[i]].astype(np.int64)
            assert (sums < 2).any(), f"{name}: source {s} target {tg[i]}: not the skipped-root case"


def test_full_size_index_file_matches_reference(built, tmp_path):
    name, c, g, idx = built
    p = tmp_path / "gpu.idx"
    idx.store_index_to_file(str(p))
    assert p.stat().st_size == c["index_bytes"]
    assert file_digest(p) == c["index_sha256"]
