"""Host-side mirror of the reference's labeler classes over the C ABI.

The reference (includes/pado_unw_unv_unp.h, pado_unw_unv_para.*.h,
pado_weighted_unv_{unp,para}.h) exposes one class per variant; the constructor
labels a rank-relabeled graph, ``order_labels`` / ``load_index_from_file``
install original ids, and ``query_distance(a, b)`` answers a pair.  The same
names, argument meanings and results are kept here; each class is backed by a
device-resident index built by the CUDA library.  Batched calls
(``query``) are added beside the per-pair one.

Errors raise :class:`PadoError` instead of the reference's print-and-exit.
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import PADO_UNWEIGHTED, PADO_WEIGHTED, PadoError, check, lib, ptr
from .graphs import CSRGraph

U8_INF = 255
I16_INF = 32767


@dataclass
class CanonicalLabels:
    """The reference's Index after order_labels, keyed by original id."""
    n: int
    K: int
    off: np.ndarray
    hub: np.ndarray
    dist: np.ndarray
    bpd: np.ndarray | None = None
    bps: np.ndarray | None = None


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


class _Index:
    kind = PADO_UNWEIGHTED

    def __init__(self, handle: C.c_void_p | None = None):
        self._h = handle

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            # a server that borrows this handle must let go of it first
            for ref in getattr(self, "_servers", ()):
                srv = ref()
                if srv is not None:
                    srv.close()
            lib.pado_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _need(self):
        if not self._h:
            raise PadoError(7, "index not built or loaded")
        return self._h

    # -- info ----------------------------------------------------------------
    def info(self) -> _lib.Info:
        inf = _lib.Info()
        check(lib.pado_get_info(self._need(), C.byref(inf)))
        return inf

    @property
    def num_v(self) -> int:
        return self.info().n

    # -- order / persistence ---------------------------------------------------
    def order_labels(self, rank2id=None, rank=None) -> None:
        """order_labels(rank2id, rank) (pado_unw_unv_unp.h:1227): queries take
        original ids from now on.  Only ``rank`` is needed."""
        if rank is None:
            if rank2id is None:
                raise ValueError("rank or rank2id required")
            r2i = _u32(rank2id)
            rank = np.empty_like(r2i)
            rank[r2i] = np.arange(len(r2i), dtype=np.uint32)
        check(lib.pado_set_order(self._need(), ptr(_u32(rank))))

    def store_index_to_file(self, filename: str, rank=None) -> None:
        """store_index_to_file (pado_unw_unv_unp.h:1120): reference format."""
        if rank is not None:
            self.order_labels(rank=rank)
        check(lib.pado_store(self._need(), str(filename).encode()))

    def load_index_from_file(self, filename: str) -> None:
        """load_index_from_file (pado_unw_unv_unp.h:1182)."""
        self.close()
        h = C.c_void_p()
        check(lib.pado_load(str(filename).encode(), self.kind, C.byref(h)))
        self._h = h

    # -- queries -------------------------------------------------------------
    def query(self, a, b) -> np.ndarray:
        """Batched query_distance over host arrays."""
        a = _u32(a)
        b = _u32(b)
        if a.shape != b.shape:
            raise ValueError("a and b must have the same shape")
        out = np.empty(a.shape, dtype=np.uint8 if self.kind == PADO_UNWEIGHTED else np.int16)
        check(lib.pado_query(self._need(), a.size, ptr(a), ptr(b), ptr(out)))
        return out

    def query_distance(self, a: int, b: int) -> int:
        return int(self.query(np.array([a]), np.array([b]))[0])

    def query_device(self, a_ptr: int, b_ptr: int, out_ptr: int, k: int, stream: int = 0) -> None:
        """Queries on device arrays (raw pointers), enqueued on ``stream``."""
        check(lib.pado_query_device(self._need(), k, C.c_void_p(a_ptr), C.c_void_p(b_ptr), C.c_void_p(out_ptr),
                                    C.c_void_p(stream)))

    # -- export --------------------------------------------------------------
    def export(self) -> CanonicalLabels:
        inf = self.info()
        n, K, tot = inf.n, inf.bp_roots, inf.num_labels
        off = np.zeros(n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.uint8 if self.kind == PADO_UNWEIGHTED else np.int16)
        bpd = np.zeros(max(n * K, 1), np.uint8) if K else None
        bps = np.zeros(max(n * K * 2, 1), np.uint64) if K else None
        check(lib.pado_export(self._need(), ptr(off), ptr(hub), ptr(dist), ptr(bpd), ptr(bps)))
        return CanonicalLabels(n, K, off, hub[:tot], dist[:tot],
                               None if bpd is None else bpd[: n * K], None if bps is None else bps[: n * K * 2])


class VertexCentricPLL(_Index):
    """Unweighted labeler (reference VertexCentricPLL<BATCH_SIZE>,
    pado_unw_unv_unp.h:42-257).

    ``VertexCentricPLL(G, rank, bp_roots=50, batch=1024)`` labels the CSR graph
    ``G`` (original ids) under vertex order ``rank`` and installs original
    ids for queries.  ``rank=None`` means ``G`` is already rank-relabeled (the
    reference's own precondition); call ``order_labels`` afterwards to query by
    original id."""
    kind = PADO_UNWEIGHTED

    def __init__(self, G: CSRGraph | None = None, rank=None, bp_roots: int = 50, batch: int = 1024):
        super().__init__()
        self.bp_roots = bp_roots
        self.batch = batch
        if G is None:
            return
        h = C.c_void_p()
        off, adj = _u64(G.off), _u32(G.adj)
        if rank is None:
            check(lib.pado_unw_build_ranked(G.n, ptr(off), ptr(adj), bp_roots, batch, C.byref(h)))
        else:
            check(lib.pado_unw_build(G.n, ptr(off), ptr(adj), ptr(_u32(rank)), bp_roots, batch, C.byref(h)))
        self._h = h

    @classmethod
    def from_edges(cls, u, v, n: int | None = None, dedupe: bool = False, bp_roots: int = 50,
                   batch: int = 1024) -> "VertexCentricPLL":
        """Edge list in, labels out, queries by original id: the reference's
        Graph -> make_rank -> id_transfer -> labeler -> order_labels sequence
        (pado.cpp main), with the graph prepared on the device
        (pado_unw_build_edges).  ``n=None`` takes max id + 1."""
        obj = cls(bp_roots=bp_roots, batch=batch)
        u, v = _u32(u), _u32(v)
        if len(u) != len(v):
            raise ValueError("u and v differ in length")
        h = C.c_void_p()
        check(lib.pado_unw_build_edges(len(u), ptr(u), ptr(v), n or 0, _lib.PADO_INGEST_DEDUPE if dedupe else 0,
                                       bp_roots, batch, C.byref(h)))
        obj._h = h
        return obj

    @classmethod
    def from_edge_file(cls, path: str, dedupe: bool = False, bp_roots: int = 50,
                       batch: int = 1024) -> "VertexCentricPLL":
        """Graph(filename) (graph.h:95-117) through labeling, parsed and
        prepared on the device (pado_build_edge_file)."""
        obj = cls(bp_roots=bp_roots, batch=batch)
        h = C.c_void_p()
        check(lib.pado_build_edge_file(str(path).encode(), PADO_UNWEIGHTED,
                                       _lib.PADO_INGEST_DEDUPE if dedupe else 0, bp_roots, batch, C.byref(h)))
        obj._h = h
        return obj

    @classmethod
    def from_labels(cls, labels: CanonicalLabels) -> "VertexCentricPLL":
        """Query-only index from canonical arrays (e.g. the reference's labels)."""
        obj = cls()
        h = C.c_void_p()
        K = labels.K
        dist = np.ascontiguousarray(labels.dist, dtype=np.uint8)
        check(lib.pado_import(PADO_UNWEIGHTED, labels.n, K, ptr(_u64(labels.off)), ptr(_u32(labels.hub)), ptr(dist),
                              ptr(np.ascontiguousarray(labels.bpd, np.uint8)) if K else None,
                              ptr(np.ascontiguousarray(labels.bps, np.uint64)) if K else None, C.byref(h)))
        obj._h = h
        return obj


class _GraphArrays:
    """Pointer arrays over many graphs for the many-graph entry points; keeps
    the per-graph numpy arrays alive while the call runs."""

    def __init__(self, graphs, ranks):
        G = len(graphs)
        if ranks is not None and len(ranks) != G:
            raise ValueError("one rank array per graph")
        self.G = G
        self.n = np.array([g.n for g in graphs], np.uint32)
        self._keep = []
        self.off = (C.c_void_p * G)()
        self.adj = (C.c_void_p * G)()
        self.rank = (C.c_void_p * G)() if ranks is not None else None
        for i, g in enumerate(graphs):
            off, adj = _u64(g.off), _u32(g.adj)
            self._keep += [off, adj]
            self.off[i] = off.ctypes.data
            self.adj[i] = adj.ctypes.data
            if ranks is not None and ranks[i] is not None:
                rk = _u32(ranks[i])
                self._keep.append(rk)
                self.rank[i] = rk.ctypes.data

    def args(self):
        return (self.G, ptr(self.n), C.cast(self.off, C.c_void_p), C.cast(self.adj, C.c_void_p),
                C.cast(self.rank, C.c_void_p) if self.rank is not None else None)


def build_many(graphs, ranks=None, bp_roots: int = 50, batch: int = 1024) -> list:
    """Label many independent graphs together (pado_unw_build_many): returns
    one VertexCentricPLL per graph, each with exactly the labels building it
    alone gives."""
    ga = _GraphArrays(graphs, ranks)
    hs = (C.c_void_p * ga.G)()
    check(lib.pado_unw_build_many(*ga.args(), bp_roots, batch, C.cast(hs, C.c_void_p)))
    out = []
    for i in range(ga.G):
        idx = VertexCentricPLL(bp_roots=bp_roots, batch=batch)
        idx._h = C.c_void_p(hs[i])
        out.append(idx)
    return out


def tune_batch(graphs, ranks=None, bp_roots: int = 50, candidates=(256, 512, 1024, 2048), sample: int = 0):
    """Pick the batch size for build_many by timing candidates on a sample of
    the graphs (pado_unw_tune_batch).  Returns (best, {candidate: ms})."""
    ga = _GraphArrays(graphs, ranks)
    cand = _u32(candidates)
    ms = np.zeros(len(cand), np.float32)
    best = C.c_uint32()
    check(lib.pado_unw_tune_batch(*ga.args(), bp_roots, ptr(cand), len(cand), sample, C.byref(best), ptr(ms)))
    return int(best.value), {int(c): float(t) for c, t in zip(cand, ms)}


_PADO_E_TIMEOUT = 6
_live_servers = weakref.WeakSet()


@atexit.register
def _close_servers():
    # stop every dispatcher thread while the interpreter and the CUDA runtime
    # are still fully alive
    for srv in list(_live_servers):
        try:
            srv.close()
        except Exception:
            pass


class Server:
    """Serving loop over device-resident label sets (pado_server_*): requests of
    any size from any thread are coalesced into mixed batches (continuous
    batching); label sets are admitted and evicted by an HBM budget.  The
    server borrows the indexes added to it until ``close()``."""

    def __init__(self, hbm_budget_bytes: int, max_batch_pairs: int = 1 << 20, slots: int = 4):
        h = C.c_void_p()
        check(lib.pado_server_create(int(hbm_budget_bytes), max_batch_pairs, slots, C.byref(h)))
        self._h = h
        self._kinds = []
        self._held = []  # borrowed indexes stay alive until the server is destroyed
        self._pending = {}
        _live_servers.add(self)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.pado_server_destroy(self._h)
            self._h = None
            self._held = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, index: _Index) -> int:
        i = C.c_uint32()
        check(lib.pado_server_add(self._h, index._need(), C.byref(i)))
        self._kinds.append(index.kind)
        self._held.append(index)
        if not hasattr(index, "_servers"):
            index._servers = []
        index._servers.append(weakref.ref(self))
        return int(i.value)

    def submit(self, index_id: int, a, b) -> int:
        """Queue a request; returns a ticket for ``wait``."""
        a, b = _u32(a), _u32(b)
        kind = self._kinds[index_id] if 0 <= index_id < len(self._kinds) else PADO_UNWEIGHTED
        out = np.empty(a.shape, np.uint8 if kind == PADO_UNWEIGHTED else np.int16)
        t = C.c_uint64()
        check(lib.pado_server_submit(self._h, index_id, a.size, ptr(a), ptr(b), ptr(out), C.byref(t)))
        self._pending[int(t.value)] = (a, b, out)
        return int(t.value)

    def wait(self, ticket: int, timeout_s: float = -1.0):
        """Results of a submitted request and its latency in seconds."""
        lat = C.c_double()
        st = lib.pado_server_wait(self._h, ticket, timeout_s, C.byref(lat))
        if st == _PADO_E_TIMEOUT:
            check(st)  # still outstanding: keep its buffers
        a, b, out = self._pending.pop(ticket)
        check(st)
        return out, float(lat.value)

    def query(self, index_id: int, a, b):
        return self.wait(self.submit(index_id, a, b))[0]

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(lib.pado_server_get_stats(self._h, C.byref(s)))
        return {f: int(getattr(s, f)) for f, _ in s._fields_ if f != "pad"}

    def replay(self, arrival_s, index_id, k, a, b, mode: int = 0):
        """Open-loop replay of a request trace (pado_server_replay).  Returns
        (out8, out16, latency_s); request i's results are out8/out16
        [pair_off[i]: pair_off[i] + k[i]] with pair_off the prefix sum of k."""
        arrival_s = np.ascontiguousarray(arrival_s, np.float64)
        index_id = _u32(index_id)
        k = _u64(k)
        pair_off = np.zeros(len(k), np.uint64)
        if len(k) > 1:
            np.cumsum(k[:-1], out=pair_off[1:])
        a, b = _u32(a), _u32(b)
        total = int(k.sum())
        out8 = np.zeros(max(total, 1), np.uint8)
        out16 = np.zeros(max(total, 1), np.int16)
        lat = np.zeros(len(k), np.float64)
        check(lib.pado_server_replay(self._h, len(k), ptr(arrival_s), ptr(index_id), ptr(k), ptr(pair_off), ptr(a),
                                     ptr(b), ptr(out8), ptr(out16), mode, ptr(lat)))
        return out8[:total], out16[:total], lat


# The OpenMP class of the reference computes the same labels
# (pado_unw_unv_para.201912311607.parallel_bp_labeling.h:42-304).
ParaVertexCentricPLL = VertexCentricPLL


class WeightedVertexCentricPLL(_Index):
    """Weighted labeler (reference WeightedVertexCentricPLL<BATCH_SIZE>,
    pado_weighted_unv_unp.h:48-236); distances are int16, 32767 = unreachable."""
    kind = PADO_WEIGHTED

    def __init__(self, G: CSRGraph | None = None, rank=None, batch: int = 512):
        super().__init__()
        self.batch = batch
        if G is None:
            return
        if G.w is None:
            raise ValueError("weighted labeling needs edge weights (G.w)")
        h = C.c_void_p()
        off, adj, w = _u64(G.off), _u32(G.adj), np.ascontiguousarray(G.w, np.uint8)
        if rank is None:
            check(lib.pado_w_build_ranked(G.n, ptr(off), ptr(adj), ptr(w), batch, C.byref(h)))
        else:
            check(lib.pado_w_build(G.n, ptr(off), ptr(adj), ptr(w), ptr(_u32(rank)), batch, C.byref(h)))
        self._h = h

    @classmethod
    def from_edges(cls, u, v, w, n: int | None = None, dedupe: bool = False,
                   batch: int = 512) -> "WeightedVertexCentricPLL":
        """Weighted edge list in, labels out, queries by original id
        (pado_w_build_edges); weights are uint8 as WeightedGraph stores them."""
        obj = cls(batch=batch)
        u, v, w = _u32(u), _u32(v), np.ascontiguousarray(w, np.uint8)
        if not (len(u) == len(v) == len(w)):
            raise ValueError("u, v and w differ in length")
        h = C.c_void_p()
        check(lib.pado_w_build_edges(len(u), ptr(u), ptr(v), ptr(w), n or 0,
                                     _lib.PADO_INGEST_DEDUPE if dedupe else 0, batch, C.byref(h)))
        obj._h = h
        return obj

    @classmethod
    def from_edge_file(cls, path: str, dedupe: bool = False, batch: int = 512) -> "WeightedVertexCentricPLL":
        """WeightedGraph(filename) (graph.h:262-290) through labeling, on the
        device (pado_build_edge_file)."""
        obj = cls(batch=batch)
        h = C.c_void_p()
        check(lib.pado_build_edge_file(str(path).encode(), PADO_WEIGHTED, _lib.PADO_INGEST_DEDUPE if dedupe else 0,
                                       0, batch, C.byref(h)))
        obj._h = h
        return obj

    @classmethod
    def from_labels(cls, labels: CanonicalLabels) -> "WeightedVertexCentricPLL":
        obj = cls()
        h = C.c_void_p()
        dist = np.ascontiguousarray(labels.dist, dtype=np.int16)
        check(lib.pado_import(PADO_WEIGHTED, labels.n, 0, ptr(_u64(labels.off)), ptr(_u32(labels.hub)), ptr(dist),
                              None, None, C.byref(h)))
        obj._h = h
        return obj


WeightedParaVertexCentricPLL = WeightedVertexCentricPLL


def graph_ingest(u, v, w=None, n: int | None = None, dedupe: bool = False):
    """Edge list (original ids) to the rank-relabeled CSR the labelers take,
    on the device (pado_graph_ingest): Graph::construct + make_rank +
    id_transfer (graph.h:125-206), degree ties by ascending id.  Returns
    ``(G_ranked, rank)``; ``rank[v]`` is the new id of vertex ``v``."""
    u, v = _u32(u), _u32(v)
    if len(u) != len(v) or (w is not None and len(w) != len(u)):
        raise ValueError("edge arrays differ in length")
    m = len(u)
    if n is None:
        n = int(max(u.max(initial=0), v.max(initial=0))) + 1 if m else 0
    wi = None if w is None else np.ascontiguousarray(w, np.uint8)
    off = np.zeros(n + 1, np.uint64)
    adj = np.zeros(max(2 * m, 1), np.uint32)
    wo = np.zeros(max(2 * m, 1), np.uint8) if wi is not None else None
    rank = np.zeros(max(n, 1), np.uint32)
    entries = C.c_uint64()
    check(lib.pado_graph_ingest(m, ptr(u), ptr(v), ptr(wi), n, _lib.PADO_INGEST_DEDUPE if dedupe else 0, ptr(off),
                                ptr(adj), ptr(wo), ptr(rank), C.byref(entries)))
    e = entries.value
    return CSRGraph(n, off, adj[:e].copy(), None if wo is None else wo[:e].copy()), rank[:n]


def _edge_arrays(u, v, n):
    u, v = _u32(u), _u32(v)
    if len(u) != len(v):
        raise ValueError("edge arrays differ in length")
    if n is None:
        n = int(max(u.max(initial=0), v.max(initial=0))) + 1 if len(u) else 0
    return u, v, len(u), n


def reduce_degree1(u, v, n: int | None = None):
    """The reference's degree-1 chain deletion
    (tools/pseudocode-delete_1-degree_vertices.cpp) on the device
    (pado_reduce_degree1).  ``n`` defaults to max id + 1, as the tool sets it.
    Returns ``(deleted, kept)``: uint8 flags per vertex and the indices of the
    input edges the tool writes, in input order."""
    u, v, m, n = _edge_arrays(u, v, n)
    deleted = np.zeros(max(n, 1), np.uint8)
    kept = np.zeros(max(m, 1), np.uint64)
    k = C.c_uint64()
    check(lib.pado_reduce_degree1(m, ptr(u), ptr(v), n, ptr(deleted), ptr(kept), C.byref(k)))
    return deleted[:n], kept[:k.value].copy()


def reduce_equivalent(u, v, n: int | None = None):
    """The reference's equivalent-vertex removal
    (distributed_version/tools/graph-convert/remove_equivalent_vertices.cpp)
    on the device (pado_reduce_equivalent).  Returns ``(redundant, new_id,
    kept, n_out)``: flags, new ids of the vertices that stay (2^32 - 1 for the
    others), indices of the kept input edges and the vertex count the tool
    writes."""
    u, v, m, n = _edge_arrays(u, v, n)
    red = np.zeros(max(n, 1), np.uint8)
    nid = np.zeros(max(n, 1), np.uint32)
    kept = np.zeros(max(m, 1), np.uint64)
    k, nout = C.c_uint64(), C.c_uint32()
    check(lib.pado_reduce_equivalent(m, ptr(u), ptr(v), n, ptr(red), ptr(nid), ptr(kept), C.byref(k),
                                     C.byref(nout)))
    return red[:n], nid[:n], kept[:k.value].copy(), int(nout.value)


def write_degree1_output(path, u, v, kept) -> None:
    """The delete_1-degree tool's output file: the kept edges as "head tail"
    lines, in input order."""
    u, v = _u32(u), _u32(v)
    with open(path, "w") as f:
        f.write("".join(f"{a} {b}\n" for a, b in zip(u[kept].tolist(), v[kept].tolist())))


def write_equivalent_output(path, u, v, new_id, kept, n_out: int) -> None:
    """The remove_equivalent_vertices tool's binary file: num_v (uint32),
    num_e (uint64), then (new_id[head], new_id[tail]) uint32 pairs."""
    u, v = _u32(u), _u32(v)
    pairs = np.stack([new_id[u[kept]], new_id[v[kept]]], 1).astype(np.uint32)
    with open(path, "wb") as f:
        f.write(np.uint32(n_out).tobytes())
        f.write(np.uint64(len(kept)).tobytes())
        f.write(pairs.tobytes())


def parse_edge_text(text: bytes, weighted: bool = False):
    """Edge-list text to arrays on the device (pado_edge_text_parse), with the
    line rules of Graph(filename) (graph.h:95-117): returns ``(u, v, w)``,
    ``w`` None when unweighted."""
    buf = np.frombuffer(text, np.uint8) if len(text) else np.zeros(1, np.uint8)
    cap = len(text) // 4 + 1
    u = np.zeros(cap, np.uint32)
    v = np.zeros(cap, np.uint32)
    w = np.zeros(cap, np.uint8) if weighted else None
    m = C.c_uint64()
    check(lib.pado_edge_text_parse(ptr(buf), len(text), int(weighted), cap, ptr(u), ptr(v), ptr(w), C.byref(m)))
    k = m.value
    return u[:k].copy(), v[:k].copy(), None if w is None else w[:k].copy()


def version() -> str:
    return lib.pado_version().decode()
