"""Generate the golden fixtures in this directory from the REFERENCE itself.

Run in a container that has the reference tree (PADO_REFERENCE_DIR, default
the mounted reference) and a working g++: the reference's own labeler classes
are compiled by oracle/build_oracle.py and driven through their public API
(constructor -> order_labels -> Index; query_distance).  Each case stores the
input graph (CSR over original ids, duplicates kept as the reference's Graph
keeps them), the vertex order, K and B, the canonical label set and a set of
(a, b, distance) query answers.  The GPU library and the oracle restatement
are both checked against these files; the tests never need the reference
tree.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from parallel_distance_oracle_gb300 import graphs as G  # noqa: E402
from oracle import orc  # noqa: E402

REF = Path(os.environ.get("PADO_REFERENCE_DIR", REPO.parent / "reference"))


def pairs_for(n: int, seed: int, k: int = 1500):
    if n <= 70:
        a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        a, b = a.ravel(), b.ravel()
    else:
        rng = np.random.Generator(np.random.PCG64(seed))
        a = rng.integers(0, n, size=k)
        b = rng.integers(0, n, size=k)
        a[:20] = b[:20]  # a == b
    # a few out-of-range ids (query answers 0 for a == b, INF otherwise)
    a = np.concatenate([a, [n, n + 3, 0]])
    b = np.concatenate([b, [n, 1 if n > 1 else 0, n + 7]])
    return a.astype(np.uint32), b.astype(np.uint32)


def unw_case(name, g, K, B, seed):
    rank = G.degree_rank(g)
    lab = orc.ref_unw_label(g, rank, K, B, mode=0)
    para = orc.ref_unw_label(g, rank, K, B, mode=1, threads=4)
    assert orc.same_unw(lab, para), f"{name}: reference seq/para disagree"
    a, b = pairs_for(g.n, seed)
    out = np.zeros(len(a), np.uint8)
    hub = lab.hub if len(lab.hub) else np.zeros(1, np.uint32)
    dist = lab.dist if len(lab.dist) else np.zeros(1, np.uint8)
    orc.ref(K).ref_unw_query(g.n, lab.off, hub, dist, np.ascontiguousarray(lab.bpd) if K else np.zeros(1, np.uint8),
                             np.ascontiguousarray(lab.bps) if K else np.zeros(1, np.uint64), len(a), a, b, out, 1)
    np.savez_compressed(HERE / f"unw_{name}.npz", kind=0, n=g.n, off=g.off, adj=g.adj, rank=rank, K=K, B=B,
                        l_off=lab.off, l_hub=lab.hub, l_dist=lab.dist, l_bpd=lab.bpd, l_bps=lab.bps,
                        qa=a, qb=b, qd=out)
    print(f"unw_{name}: n={g.n} m={g.m_directed} K={K} B={B} labels={len(lab.hub)}")


def w_case(name, g, B, seed):
    rank = G.degree_rank(g)
    lab = orc.ref_w_label(g, rank, B, mode=0)
    para = orc.ref_w_label(g, rank, B, mode=1, threads=4)
    assert orc.same_w(lab, para), f"{name}: reference seq/para disagree"
    a, b = pairs_for(g.n, seed)
    out = np.zeros(len(a), np.int16)
    hub = lab.hub if len(lab.hub) else np.zeros(1, np.uint32)
    dist = lab.dist if len(lab.dist) else np.zeros(1, np.int16)
    orc.ref(50).ref_w_query(g.n, lab.off, hub, dist, len(a), a, b, out, 1)
    np.savez_compressed(HERE / f"w_{name}.npz", kind=1, n=g.n, off=g.off, adj=g.adj, w=g.w, rank=rank, K=0, B=B,
                        l_off=lab.off, l_hub=lab.hub, l_dist=lab.dist, qa=a, qb=b, qd=out)
    print(f"w_{name}: n={g.n} m={g.m_directed} B={B} labels={len(lab.hub)}")


def main():
    for p in list(HERE.glob("unw_*.npz")) + list(HERE.glob("w_*.npz")):
        p.unlink()
    tools = REF / "tools"
    # the reference's own fixture graphs
    unw_case("ref_edgelist_k50", G.read_edge_list(str(tools / "edgelist.in")), 50, 1024, 1)
    unw_case("ref_edgelist_k4_b8", G.read_edge_list(str(tools / "edgelist.in")), 4, 8, 2)
    unw_case("ref_deleted_k2_b8", G.read_edge_list(str(tools / "deleted_graph.in")), 2, 8, 3)
    unw_case("ref_rectangle_k0_b8", G.read_edge_list(str(tools / "rectangle.in")), 0, 8, 4)
    for nm in ["weighted_edgelist", "1_w_edgelist", "7_w_edgelist", "triangle", "rectangle"]:
        w_case(f"ref_{nm}_b8", G.read_edge_list(str(tools / f"{nm}.in"), weighted=True), 8, 5)
    w_case("ref_weighted_edgelist_b512", G.read_edge_list(str(tools / "weighted_edgelist.in"), weighted=True), 512, 6)
    # seeded synthetic graphs
    unw_case("rmat9_k50_b64", G.rmat(9, 8, 7), 50, 64, 10)
    unw_case("rmat10_k64_b128", G.rmat(10, 8, 8), 64, 128, 11)
    unw_case("rmat10_k16_b32", G.rmat(10, 16, 9), 16, 32, 12)
    unw_case("er600_k8_b64", G.erdos_renyi(600, 6, 13), 8, 64, 13)
    unw_case("grid500_k10_b16", G.grid_with_shortcuts(500, 0.02, 14), 10, 16, 14)
    unw_case("path90_k2_b16", G.path_graph(90), 2, 16, 15)
    star = G.csr_from_edges(60, np.zeros(59, np.int64), np.arange(1, 60))
    unw_case("star60_k1_b8", star, 1, 8, 16)
    # disconnected: two R-MAT pieces plus isolated vertices
    g1, g2 = G.rmat(8, 4, 17), G.rmat(7, 4, 18)
    u1, v1 = np.repeat(np.arange(g1.n), np.diff(g1.off).astype(np.int64)), g1.adj.astype(np.int64)
    u2, v2 = np.repeat(np.arange(g2.n), np.diff(g2.off).astype(np.int64)), g2.adj.astype(np.int64) + g1.n
    dis = G.csr_from_edges(g1.n + g2.n + 40, np.concatenate([u1, u2 + g1.n]), np.concatenate([v1, v2]))
    unw_case("disconnected_k8_b32", dis, 8, 32, 19)
    # raw input with duplicate edges and self-loops, kept as Graph keeps them
    rng = np.random.Generator(np.random.PCG64(20))
    ru = rng.integers(0, 150, 700)
    rv = rng.integers(0, 150, 700)
    rv[:30] = ru[:30]
    ru = np.concatenate([ru, ru[100:160]])
    rv = np.concatenate([rv, rv[100:160]])
    unw_case("dups_selfloops_k6_b16", G.csr_keep_duplicates(150, ru, rv), 6, 16, 20)
    # weighted synthetic
    w_case("rmat9_w100_b64", G.rmat(9, 8, 21, weights=(1, 100)), 64, 21)
    w_case("rmat10_w7_b128", G.rmat(10, 8, 22, weights=(1, 7)), 128, 22)
    gg = G.grid_with_shortcuts(400, 0.02, 23)
    gg.w = np.random.Generator(np.random.PCG64(23)).integers(1, 4, gg.m_directed).astype(np.uint8)
    # symmetric weights: give both directions of each edge the same weight
    wsym = _symmetric_weights(gg, seed=23, lo=1, hi=3)
    gg.w = wsym
    w_case("grid400_w3_b32", gg, 32, 23)
    ww = rng.integers(1, 60, 300)
    wu = rng.integers(0, 120, 300)
    wv = rng.integers(0, 120, 300)
    w_case("dups_w60_b16", G.csr_keep_duplicates(120, wu, wv, ww), 16, 24)


def _symmetric_weights(g, seed, lo, hi):
    """Per undirected edge weight, the same in both CSR directions."""
    rng = np.random.Generator(np.random.PCG64(seed))
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    dst = g.adj.astype(np.int64)
    key = np.minimum(src, dst) * g.n + np.maximum(src, dst)
    uniq, inv = np.unique(key, return_inverse=True)
    wu = rng.integers(lo, hi + 1, len(uniq))
    return wu[inv].astype(np.uint8)


if __name__ == "__main__" and len(sys.argv) == 1:
    main()


# ---------------------------------------------------------------------------
# Index files written by the reference itself: for a few of the cases above,
# the reference's sequential labeler (VertexCentricPLL<B> /
# WeightedVertexCentricPLL<B>) writes its index with store_index_to_file
# (pado_unw_unv_unp.h:1120-1180, pado_weighted_unv_unp.h:1639-1676), and its
# load_index_from_file (pado_unw_unv_unp.h:1182-1224 with the root count read
# into a local; pado_weighted_unv_unp.h:1678-1711) reads the file back and
# answers the case's query pairs.  Stored: the file's bytes and those answers.
# Run:  python tests/golden/make_golden.py --index-files
# ---------------------------------------------------------------------------
INDEX_FILE_CASES = ["unw_ref_edgelist_k50", "unw_rmat9_k50_b64", "unw_rmat10_k64_b128", "w_ref_weighted_edgelist_b512",
                    "w_rmat9_w100_b64", "w_rmat10_w7_b128"]


def index_files():
    import tempfile
    for p in HERE.glob("idxfile_*.npz"):
        p.unlink()
    tmp = Path(tempfile.mkdtemp())
    for case in INDEX_FILE_CASES:
        z = np.load(HERE / f"{case}.npz")
        weighted = int(z["kind"]) == 1
        g = G.CSRGraph(n=int(z["n"]), off=z["off"], adj=z["adj"], w=z["w"] if weighted else None)
        rank, K, B = z["rank"], int(z["K"]), int(z["B"])
        path = tmp / f"{case}.idx"
        if weighted:
            orc.ref_w_store(g, rank, B, path)
        else:
            orc.ref_unw_store(g, rank, K, B, path)
        loaded = orc.ref_load_query(path, z["qa"], z["qb"], weighted=weighted, K=K)
        # the reloaded index answers as the labeler's own index does
        assert np.array_equal(loaded, z["qd"]), f"{case}: reloaded reference index answers differently"
        raw = np.frombuffer(path.read_bytes(), np.uint8)
        np.savez_compressed(HERE / f"idxfile_{case}.npz", case=case, raw=raw, qa=z["qa"], qb=z["qb"], qd=loaded)
        print(f"idxfile_{case}: {len(raw)} bytes")


if __name__ == "__main__" and sys.argv[1:2] == ["--index-files"]:
    index_files()


# ---------------------------------------------------------------------------
# Full-size digests: the configs' own graphs are too large to store, so the
# reference's canonical label set for each is reduced to a SHA-256 digest of
# (off, hub, dist[, bp_dist, bp_sets]) in that order, little-endian, plus the
# label count.  Run:  python tests/golden/make_golden.py --digests
# ---------------------------------------------------------------------------
DIGEST_CASES = {
    # R-MAT s14 ef8, degree order, K=50, B=1024
    "rmat14_k50_b1024": dict(kind="unw", scale=14, ef=8, seed=1, K=50, B=1024),
    # R-MAT s20 ef16, degree order, K=64, B=1024
    "rmat20_k64_b1024": dict(kind="unw", scale=20, ef=16, seed=2, K=64, B=1024),
    # weighted R-MAT s18 ef8, weights U[1,100], degree order, B=512
    "wrmat18_b512": dict(kind="w", scale=18, ef=8, seed=3, K=0, B=512),
}


def label_digest(kind, off, hub, dist, bpd=None, bps=None):
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(hub, np.uint32).tobytes())
    h.update(np.ascontiguousarray(dist, np.uint8 if kind == "unw" else np.int16).tobytes())
    if bpd is not None and len(bpd):
        h.update(np.ascontiguousarray(bpd, np.uint8).tobytes())
        h.update(np.ascontiguousarray(bps, np.uint64).tobytes())
    return h.hexdigest()


def digests():
    import json
    import os as _os
    out = {}
    for name, c in DIGEST_CASES.items():
        w = (1, 100) if c["kind"] == "w" else None
        g = G.rmat(c["scale"], c["ef"], c["seed"], weights=w)
        rank = G.degree_rank(g)
        threads = _os.cpu_count() or 1
        if c["kind"] == "unw":
            lab = orc.ref_unw_label(g, rank, c["K"], c["B"], mode=1, threads=threads)
            dg = label_digest("unw", lab.off, lab.hub, lab.dist, lab.bpd, lab.bps)
        else:
            lab = orc.ref_w_label(g, rank, c["B"], mode=1, threads=threads)
            dg = label_digest("w", lab.off, lab.hub, lab.dist)
        out[name] = dict(c, labels=int(len(lab.hub)), sha256=dg, reference_seconds=round(lab.seconds, 2),
                         reference_threads=threads)
        print(name, out[name], flush=True)
    (HERE / "full_size_digests.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__" and sys.argv[1:2] == ["--digests"]:
    digests()


# Query answers and index files at full size, added to the same JSON:
#   queries -- count, seed and SHA-256 of the answers (uint8 / int16,
#     little-endian) of the reference's query_distance (pado_unw_unv_unp.h:
#     1312-1445; weighted pado_weighted_unv_unp.h:1782-1900) over its own
#     labels, for the workload's query pairs (graphs.random_pairs(n, count,
#     seed));
#   index_sha256 / index_bytes -- the file the reference's sequential labeler
#     writes with its own store_index_to_file (the OpenMP unweighted class's
#     writer writes nothing: its body is commented out).
# Run:  python tests/golden/make_golden.py --digests-extra [names...]
QUERY_SETS = {"rmat14_k50_b1024": (100_000, 11), "rmat20_k64_b1024": (10_000_000, 12), "wrmat18_b512": (1_000_000, 13)}


def _sha_file(path):
    import hashlib
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 24), b""):
            h.update(chunk)
    return h.hexdigest()


def digests_extra(names):
    import hashlib
    import json
    import os as _os
    import tempfile
    path = HERE / "full_size_digests.json"
    out = json.loads(path.read_text())
    threads = _os.cpu_count() or 1
    for name in names:
        c = out[name]
        w = (1, 100) if c["kind"] == "w" else None
        g = G.rmat(c["scale"], c["ef"], c["seed"], weights=w)
        rank = G.degree_rank(g)
        nq, qseed = QUERY_SETS[name]
        qa, qb = G.random_pairs(g.n, nq, qseed)
        if c["kind"] == "unw":
            lab = orc.ref_unw_label(g, rank, c["K"], c["B"], mode=1, threads=threads)
            assert label_digest("unw", lab.off, lab.hub, lab.dist, lab.bpd, lab.bps) == c["sha256"]
            ans = np.zeros(nq, np.uint8)
            orc.ref(c["K"]).ref_unw_query(g.n, lab.off, lab.hub, lab.dist, np.ascontiguousarray(lab.bpd),
                                          np.ascontiguousarray(lab.bps), nq, qa, qb, ans, threads)
        else:
            lab = orc.ref_w_label(g, rank, c["B"], mode=1, threads=threads)
            assert label_digest("w", lab.off, lab.hub, lab.dist) == c["sha256"]
            ans = np.zeros(nq, np.int16)
            orc.ref(50).ref_w_query(g.n, lab.off, lab.hub, lab.dist, nq, qa, qb, ans, threads)
        del lab
        c["queries"] = dict(count=nq, seed=qseed, sha256=hashlib.sha256(ans.tobytes()).hexdigest(),
                            unreachable=int((ans == (255 if c["kind"] == "unw" else 32767)).sum()))
        print(name, "queries", c["queries"], flush=True)
        path.write_text(json.dumps(out, indent=1) + "\n")
        tmp = Path(tempfile.mkdtemp()) / "index.idx"
        if c["kind"] == "unw":
            orc.ref_unw_store(g, rank, c["K"], c["B"], tmp)
        else:
            orc.ref_w_store(g, rank, c["B"], tmp)
        c["index_sha256"] = _sha_file(tmp)
        c["index_bytes"] = tmp.stat().st_size
        tmp.unlink()
        print(name, "index", c["index_sha256"], c["index_bytes"], flush=True)
        path.write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__" and sys.argv[1:2] == ["--digests-extra"]:
    digests_extra([a for a in sys.argv[2:] if not a.startswith("-")] or list(QUERY_SETS))
