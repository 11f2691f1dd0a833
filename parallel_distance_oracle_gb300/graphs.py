"""Seeded synthetic graphs, vertex orders and query pairs.

The reference benchmarks on downloaded SNAP/KONECT graphs
(scripts/get_datasets.sh); those are not available here, so seeded synthetic
graphs with the benchmark's shapes stand in for them.  Everything is numpy with
PCG64 streams, so the same seed gives the same graph on x86 and Arm.

Graphs are returned as an undirected CSR over ORIGINAL vertex ids with both
directions stored, duplicates and self-loops removed (the reference's Graph
keeps duplicates, graph.h:125-153, so callers must not feed it any), and
neighbour lists in ascending id order.  The labelers relabel by rank themselves
(graph.h:176-206 semantics).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSRGraph:
    n: int
    off: np.ndarray            # uint64[n + 1]
    adj: np.ndarray            # uint32[off[n]]
    w: np.ndarray | None = None  # uint8[off[n]] for weighted graphs

    @property
    def m_directed(self) -> int:
        return int(self.off[-1])

    def degrees(self) -> np.ndarray:
        return np.diff(self.off).astype(np.int64)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def csr_from_edges(n: int, u: np.ndarray, v: np.ndarray, w: np.ndarray | None = None) -> CSRGraph:
    """Undirected CSR from an edge list: self-loops dropped, duplicates merged
    (the first weight of a duplicated pair wins), both directions stored."""
    u = np.asarray(u, dtype=np.uint64)
    v = np.asarray(v, dtype=np.uint64)
    keep = u != v
    u, v = u[keep], v[keep]
    if w is not None:
        w = np.asarray(w, dtype=np.uint8)[keep]
    lo = np.minimum(u, v)
    hi = np.maximum(u, v)
    key = lo * np.uint64(n) + hi
    key, first = np.unique(key, return_index=True)
    lo = key // np.uint64(n)
    hi = key % np.uint64(n)
    ww = w[first] if w is not None else None
    src = np.concatenate([lo, hi])
    dst = np.concatenate([hi, lo])
    order = np.lexsort((dst, src))
    src = src[order]
    dst = dst[order]
    deg = np.bincount(src.astype(np.int64), minlength=n)
    off = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(deg, out=off[1:])
    wd = None
    if ww is not None:
        wd = np.concatenate([ww, ww])[order].astype(np.uint8)
    return CSRGraph(n=n, off=off, adj=dst.astype(np.uint32), w=wd)


def rmat(scale: int, edge_factor: int, seed: int, a: float = 0.57, b: float = 0.19,
         c: float = 0.19, weights: tuple[int, int] | None = None) -> CSRGraph:
    """R-MAT graph on n = 2**scale vertices from n * edge_factor samples.

    Per sample and per bit level, quadrant a/b/c/d (d = 1 - a - b - c) picks the
    (row, column) bit pair (0,0)/(0,1)/(1,0)/(1,1).  Self-loops are dropped and
    the result symmetrised and deduplicated; isolated vertices are kept.  With
    ``weights=(lo, hi)``, each undirected edge gets a uniform integer weight in
    [lo, hi] drawn from the same stream after the structure."""
    return csr_from_edges(*rmat_edges(scale, edge_factor, seed, a, b, c, weights))


def rmat_edges(scale: int, edge_factor: int, seed: int, a: float = 0.57, b: float = 0.19,
               c: float = 0.19, weights: tuple[int, int] | None = None):
    """The raw samples behind :func:`rmat`, before cleaning: ``(n, u, v, w)``
    with self-loops and repeats still in (``w`` None without weights)."""
    n = 1 << scale
    m = n * edge_factor
    rng = _rng(seed)
    u = np.zeros(m, dtype=np.uint64)
    v = np.zeros(m, dtype=np.uint64)
    ab, abc = a + b, a + b + c
    for bit in range(scale):
        r = rng.random(m)
        ubit = (r >= ab).astype(np.uint64)
        vbit = (((r >= a) & (r < ab)) | (r >= abc)).astype(np.uint64)
        u |= ubit << np.uint64(bit)
        v |= vbit << np.uint64(bit)
    w = None
    if weights is not None:
        w = rng.integers(weights[0], weights[1] + 1, size=m, dtype=np.int64).astype(np.uint8)
    return n, u, v, w


def erdos_renyi(n: int, avg_degree: float, seed: int) -> CSRGraph:
    """G(n, m) with m = n * avg_degree / 2 uniformly drawn pairs (self-loops and
    repeats dropped)."""
    rng = _rng(seed)
    m = int(round(n * avg_degree / 2))
    u = rng.integers(0, n, size=m, dtype=np.int64)
    v = rng.integers(0, n, size=m, dtype=np.int64)
    return csr_from_edges(n, u, v)


def grid_with_shortcuts(n: int, frac: float, seed: int) -> CSRGraph:
    """ceil(sqrt n) columns, row-major, truncated to n vertices, 4-neighbour
    edges, plus frac * (grid edges) uniformly random long-range edges."""
    rng = _rng(seed)
    cols = int(np.ceil(np.sqrt(n)))
    ids = np.arange(n, dtype=np.int64)
    right = ids[(ids % cols != cols - 1) & (ids + 1 < n)]
    down = ids[ids + cols < n]
    u = np.concatenate([right, down])
    v = np.concatenate([right + 1, down + cols])
    k = int(round(frac * len(u)))
    su = rng.integers(0, n, size=k, dtype=np.int64)
    sv = rng.integers(0, n, size=k, dtype=np.int64)
    return csr_from_edges(n, np.concatenate([u, su]), np.concatenate([v, sv]))


def reduction_edges(n: int, seed: int, iso_path_max: int = 4):
    """An edge list ``(u, v)`` (uint32, ids < n, input order) rich in what the
    reference's reduction tools remove: a sparse random core on half the
    vertices, pendant paths of 1-6 vertices and pendant stars hung on it,
    cliques of 3-5 vertices joined to the core by one member (the others have
    equal closed neighbourhoods), isolated paths of 2..iso_path_max vertices,
    and about 1% repeated edges and 0.5% self-loops.  Ids are shuffled and
    the edges put in random order.  (On an isolated path of four or more
    vertices the reference's degree-1 tool can walk for ever, depending on
    the edge order; a core vertex left without core edges turns the pendant
    paths hung on it into such a path too.)"""
    rng = _rng(seed)
    core = max(n // 2, 2)
    us = list(rng.integers(0, core, 2 * core))
    vs = list(rng.integers(0, core, 2 * core))
    nxt = core

    def add(a, b):
        us.append(a)
        vs.append(b)

    while nxt < n:
        kind = rng.random()
        if kind < 0.45:  # pendant path
            prev = int(rng.integers(0, core))
            for _ in range(int(rng.integers(1, 7))):
                if nxt >= n:
                    break
                add(prev, nxt)
                prev, nxt = nxt, nxt + 1
        elif kind < 0.6:  # pendant star
            hub = int(rng.integers(0, core))
            for _ in range(int(rng.integers(2, 6))):
                if nxt >= n:
                    break
                add(hub, nxt)
                nxt += 1
        elif kind < 0.85:  # clique with one member on the core
            k = min(int(rng.integers(3, 6)), n - nxt)
            mem = list(range(nxt, nxt + k))
            nxt += k
            for i in range(k):
                for j in range(i + 1, k):
                    add(mem[i], mem[j])
            add(mem[0], int(rng.integers(0, core)))
        else:  # isolated path (a single edge when it has two vertices)
            k = min(int(rng.integers(2, iso_path_max + 1)), n - nxt)
            for i in range(k - 1):
                add(nxt + i, nxt + i + 1)
            nxt += k
    u = np.array(us, dtype=np.int64)
    v = np.array(vs, dtype=np.int64)
    rep = rng.integers(0, len(u), size=max(len(u) // 100, 1))
    loops = rng.integers(0, n, size=max(n // 200, 1))
    u = np.concatenate([u, u[rep], loops])
    v = np.concatenate([v, v[rep], loops])
    perm = rng.permutation(n)
    order = rng.permutation(len(u))
    return perm[u[order]].astype(np.uint32), perm[v[order]].astype(np.uint32)


def path_graph(n: int) -> CSRGraph:
    i = np.arange(n - 1, dtype=np.int64)
    return csr_from_edges(n, i, i + 1)


def degree_rank(g: CSRGraph) -> np.ndarray:
    """rank[v] = position of v when vertices are sorted by degree descending,
    ties broken by ascending id (rank 0 = most important).  This is the
    deterministic stand-in for Graph::make_rank (graph.h:156-174), whose
    rand()-based tiebreak is not reproducible across hosts."""
    deg = g.degrees()
    order = np.lexsort((np.arange(g.n), -deg))
    rank = np.empty(g.n, dtype=np.uint32)
    rank[order] = np.arange(g.n, dtype=np.uint32)
    return rank


def random_pairs(n: int, k: int, seed: int, distinct: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """k uniform random (a, b) pairs, a != b when ``distinct``."""
    rng = _rng(seed)
    a = rng.integers(0, n, size=k, dtype=np.int64)
    b = rng.integers(0, n, size=k, dtype=np.int64)
    if distinct and n > 1:
        bad = a == b
        while bad.any():
            b[bad] = rng.integers(0, n, size=int(bad.sum()), dtype=np.int64)
            bad = a == b
    return a.astype(np.uint32), b.astype(np.uint32)


def csr_keep_duplicates(n: int, u, v, w=None) -> CSRGraph:
    """CSR exactly as the reference's Graph::construct builds it
    (graph.h:125-153, weighted :281-309): for each input edge (u, v) in order,
    v is appended to u's list and u to v's; duplicates and self-loops are
    kept (a self-loop appears twice in its vertex's list)."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    k = len(u)
    src = np.empty(2 * k, dtype=np.int64)
    dst = np.empty(2 * k, dtype=np.int64)
    src[0::2], dst[0::2] = u, v
    src[1::2], dst[1::2] = v, u
    order = np.argsort(src, kind="stable")
    deg = np.bincount(src, minlength=n)
    off = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(deg, out=off[1:])
    wd = None
    if w is not None:
        ww = np.empty(2 * k, dtype=np.uint8)
        ww[0::2] = ww[1::2] = np.asarray(w, dtype=np.int64).astype(np.uint8)
        wd = ww[order]
    return CSRGraph(n=n, off=off, adj=dst[order].astype(np.uint32), w=wd)


def read_edge_list(path: str, weighted: bool = False) -> CSRGraph:
    """Text edge list as the reference reads it (graph.h:95-117): lines
    starting with '#' or '%' are skipped; 'u v' or 'u v w'; n = max id + 1;
    weights are cast to uint8 (graph.h:300)."""
    us, vs, ws = [], [], []
    with open(path) as f:
        for line in f:
            if not line.strip() or line[0] in "#%":
                continue
            parts = line.split()
            us.append(int(parts[0]))
            vs.append(int(parts[1]))
            if weighted:
                ws.append(int(parts[2]) & 0xFF)
    n = max(max(us), max(vs)) + 1 if us else 0
    return csr_keep_duplicates(n, us, vs, ws if weighted else None)
