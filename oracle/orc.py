"""ctypes wrappers over the oracle (liboracle.so) and the reference driver
(oracle/_ref/libpado_ref_k*.so).  TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import build_oracle as _b

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i16p = np.ctypeslib.ndpointer(np.int16, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


@dataclass
class UnwLabels:
    """Canonical unweighted label set keyed by ORIGINAL id (order_labels form):
    per vertex the (rank hub, dist) pairs sorted by hub, plus K BP rows."""
    n: int
    K: int
    off: np.ndarray    # uint64[n+1]
    hub: np.ndarray    # uint32
    dist: np.ndarray   # uint8
    bpd: np.ndarray    # uint8[n*K]
    bps: np.ndarray    # uint64[n*K*2]  (S^-1, S^0)
    seconds: float = 0.0
    stats: dict | None = None


@dataclass
class WLabels:
    n: int
    off: np.ndarray
    hub: np.ndarray
    dist: np.ndarray   # int16
    seconds: float = 0.0
    stats: dict | None = None


UNW_STATS = ["batches", "levels", "head_visits", "edges_scanned", "pairs_offered", "bp_checks",
             "bp_pruned", "dist_checks", "dist_entries", "labels_added", "root_rows", "cand_vertices"]
W_STATS = ["batches", "rounds", "edges_scanned", "relax_tries", "relax_accepted", "checks",
           "check_entries", "temp_labels", "filtered", "labels_added"]

_port = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        so = _b.build_port()
        lib = C.CDLL(str(so))
        lib.orc_unw_build.restype = C.c_void_p
        lib.orc_unw_build.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_uint32]
        lib.orc_unw_num_labels.restype = C.c_uint64
        lib.orc_unw_num_labels.argtypes = [C.c_void_p]
        lib.orc_unw_export.argtypes = [C.c_void_p, _u64p, _u32p, _u8p, _u8p, _u64p]
        lib.orc_unw_stats.argtypes = [C.c_void_p, _u64p]
        lib.orc_unw_query.argtypes = [C.c_void_p, C.c_uint64, _u32p, _u32p, _u8p]
        lib.orc_unw_query_arrays.argtypes = [C.c_uint32, C.c_uint32, _u64p, _u32p, _u8p, _u8p, _u64p,
                                             C.c_uint64, _u32p, _u32p, _u8p]
        lib.orc_unw_free.argtypes = [C.c_void_p]
        lib.orc_unw_store.restype = C.c_int
        lib.orc_unw_store.argtypes = [C.c_void_p, C.c_char_p]
        lib.orc_w_build.restype = C.c_void_p
        lib.orc_w_build.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, _u32p, C.c_uint32, C.c_uint32]
        lib.orc_w_num_labels.restype = C.c_uint64
        lib.orc_w_num_labels.argtypes = [C.c_void_p]
        lib.orc_w_export.argtypes = [C.c_void_p, _u64p, _u32p, _i16p]
        lib.orc_w_stats.argtypes = [C.c_void_p, _u64p]
        lib.orc_w_query.argtypes = [C.c_void_p, C.c_uint64, _u32p, _u32p, _i16p]
        lib.orc_w_query_arrays.argtypes = [C.c_uint32, _u64p, _u32p, _i16p, C.c_uint64, _u32p, _u32p, _i16p]
        lib.orc_w_free.argtypes = [C.c_void_p]
        lib.orc_w_store.restype = C.c_int
        lib.orc_w_store.argtypes = [C.c_void_p, C.c_char_p]
        lib.orc_unw_prefix.restype = C.c_double
        lib.orc_unw_prefix.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_double)]
        lib.orc_bfs.argtypes = [C.c_uint32, _u64p, _u32p, C.c_uint32, _u8p]
        lib.orc_dijkstra.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, C.c_uint32, _i32p]
        lib.orc_graph_ingest.restype = C.c_int
        lib.orc_graph_ingest.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int,
                                         _u64p, _u32p, C.c_void_p, _u32p, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint32)]
        lib.orc_edge_text_parse.restype = C.c_uint64
        lib.orc_edge_text_parse.argtypes = [C.c_char_p, C.c_uint64, C.c_int, C.c_uint64, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
        lib.orc_reduce_degree1.restype = C.c_int
        lib.orc_reduce_degree1.argtypes = [C.c_uint64, _u32p, _u32p, C.c_uint32, _u8p, _u64p,
                                           C.POINTER(C.c_uint64), C.POINTER(C.c_int)]
        lib.orc_reduce_equivalent.restype = C.c_int
        lib.orc_reduce_equivalent.argtypes = [C.c_uint64, _u32p, _u32p, C.c_uint32, _u8p, _u32p, _u64p,
                                              C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        _port = lib
    return _port


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def unw_label(g, rank, K: int, B: int) -> UnwLabels:
    """Oracle unweighted labeling of CSR graph ``g`` under vertex order ``rank``."""
    lib = port()
    h = lib.orc_unw_build(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(rank, np.uint32), K, B)
    try:
        tot = lib.orc_unw_num_labels(h)
        off = np.zeros(g.n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.uint8)
        bpd = np.zeros(max(g.n * K, 1), np.uint8)
        bps = np.zeros(max(g.n * K * 2, 1), np.uint64)
        lib.orc_unw_export(h, off, hub, dist, bpd, bps)
        st = np.zeros(len(UNW_STATS), np.uint64)
        lib.orc_unw_stats(h, st)
    finally:
        lib.orc_unw_free(h)
    return UnwLabels(g.n, K, off, hub[:tot], dist[:tot], bpd[: g.n * K], bps[: g.n * K * 2],
                     stats=dict(zip(UNW_STATS, map(int, st))))


def w_label(g, rank, B: int, mode: int = 0) -> WLabels:
    lib = port()
    h = lib.orc_w_build(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(g.w, np.uint8),
                        _c(rank, np.uint32), B, mode)
    try:
        tot = lib.orc_w_num_labels(h)
        off = np.zeros(g.n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.int16)
        lib.orc_w_export(h, off, hub, dist)
        st = np.zeros(len(W_STATS), np.uint64)
        lib.orc_w_stats(h, st)
    finally:
        lib.orc_w_free(h)
    return WLabels(g.n, off, hub[:tot], dist[:tot], stats=dict(zip(W_STATS, map(int, st))))


def unw_query(lab: UnwLabels, a, b) -> np.ndarray:
    a = _c(a, np.uint32)
    b = _c(b, np.uint32)
    out = np.zeros(len(a), np.uint8)
    hub = lab.hub if len(lab.hub) else np.zeros(1, np.uint32)
    dist = lab.dist if len(lab.dist) else np.zeros(1, np.uint8)
    port().orc_unw_query_arrays(lab.n, lab.K, _c(lab.off, np.uint64), _c(hub, np.uint32),
                                _c(dist, np.uint8), _c(lab.bpd, np.uint8), _c(lab.bps, np.uint64),
                                len(a), a, b, out)
    return out


def w_query(lab: WLabels, a, b) -> np.ndarray:
    a = _c(a, np.uint32)
    b = _c(b, np.uint32)
    out = np.zeros(len(a), np.int16)
    hub = lab.hub if len(lab.hub) else np.zeros(1, np.uint32)
    dist = lab.dist if len(lab.dist) else np.zeros(1, np.int16)
    port().orc_w_query_arrays(lab.n, _c(lab.off, np.uint64), _c(hub, np.uint32), _c(dist, np.int16),
                              len(a), a, b, out)
    return out


def bfs(g, src: int) -> np.ndarray:
    out = np.zeros(g.n, np.uint8)
    port().orc_bfs(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), src, out)
    return out


def dijkstra(g, src: int) -> np.ndarray:
    out = np.zeros(g.n, np.int32)
    port().orc_dijkstra(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(g.w, np.uint8), src, out)
    return out


# --------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built).
# --------------------------------------------------------------------------
_refs: dict[int, C.CDLL] = {}


def ref_available(K: int = 50) -> bool:
    return _b.ref_so(K).exists() or bool(_b.build_reference() and _b.ref_so(K).exists())


def ref(K: int = 50) -> C.CDLL:
    if K not in _refs:
        so = _b.ref_so(K)
        if not so.exists():
            _b.build_reference(sizes=(K,))
        if not so.exists():
            raise FileNotFoundError(f"reference driver {so} not built")
        lib = C.CDLL(str(so))
        lib.ref_set_threads.argtypes = [C.c_int]
        lib.ref_unw_build.restype = C.c_void_p
        lib.ref_unw_build.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_int]
        lib.ref_unw_num_labels.restype = C.c_uint64
        lib.ref_unw_num_labels.argtypes = [C.c_void_p]
        lib.ref_unw_seconds.restype = C.c_double
        lib.ref_unw_seconds.argtypes = [C.c_void_p]
        lib.ref_unw_export.argtypes = [C.c_void_p, _u64p, _u32p, _u8p, _u8p, _u64p]
        lib.ref_unw_free.argtypes = [C.c_void_p]
        lib.ref_w_build.restype = C.c_void_p
        lib.ref_w_build.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, _u32p, C.c_uint32, C.c_int]
        lib.ref_w_num_labels.restype = C.c_uint64
        lib.ref_w_num_labels.argtypes = [C.c_void_p]
        lib.ref_w_seconds.restype = C.c_double
        lib.ref_w_seconds.argtypes = [C.c_void_p]
        lib.ref_w_export.argtypes = [C.c_void_p, _u64p, _u32p, _i16p]
        lib.ref_w_free.argtypes = [C.c_void_p]
        lib.ref_unw_prefix.restype = C.c_double
        lib.ref_unw_prefix.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_double)]
        lib.ref_unw_query.restype = C.c_double
        lib.ref_unw_query.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, _u8p, _u64p, C.c_uint64,
                                      _u32p, _u32p, _u8p, C.c_int]
        lib.ref_w_query.restype = C.c_double
        lib.ref_w_query.argtypes = [C.c_uint32, _u64p, _u32p, _i16p, C.c_uint64, _u32p, _u32p,
                                    _i16p, C.c_int]
        lib.ref_unw_store.restype = C.c_int
        lib.ref_unw_store.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_char_p]
        lib.ref_w_store.restype = C.c_int
        lib.ref_w_store.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, _u32p, C.c_uint32, C.c_char_p]
        lib.ref_unw_load_query.restype = C.c_int64
        lib.ref_unw_load_query.argtypes = [C.c_char_p, C.c_uint64, _u32p, _u32p, _u8p]
        lib.ref_w_load_query.restype = C.c_int64
        lib.ref_w_load_query.argtypes = [C.c_char_p, C.c_uint64, _u32p, _u32p, _i16p]
        lib.ref_graph_read.restype = C.c_void_p
        lib.ref_graph_read.argtypes = [C.c_char_p, C.c_int]
        lib.ref_graph_make.restype = C.c_void_p
        lib.ref_graph_make.argtypes = [C.c_uint64, _u32p, _u32p, C.c_void_p]
        lib.ref_graph_n.restype = C.c_uint32
        lib.ref_graph_n.argtypes = [C.c_void_p]
        lib.ref_graph_entries.restype = C.c_uint64
        lib.ref_graph_entries.argtypes = [C.c_void_p]
        lib.ref_graph_degrees.argtypes = [C.c_void_p, _u32p]
        lib.ref_graph_transfer.argtypes = [C.c_void_p, _u32p, _u64p, _u32p, C.c_void_p]
        lib.ref_graph_free.argtypes = [C.c_void_p]
        _refs[K] = lib
    return _refs[K]


def _ranked_from_ref(lib, h, weighted: bool):
    """Degree order with ascending-id ties over the reference Graph's own
    degrees, then its id_transfer; returns (CSRGraph, rank)."""
    n = lib.ref_graph_n(h)
    e = lib.ref_graph_entries(h)
    deg = np.zeros(max(n, 1), np.uint32)
    lib.ref_graph_degrees(h, deg)
    deg = deg[:n]
    order = np.lexsort((np.arange(n), -deg.astype(np.int64)))
    rank = np.empty(n, np.uint32)
    rank[order] = np.arange(n, dtype=np.uint32)
    off = np.zeros(n + 1, np.uint64)
    adj = np.zeros(max(e, 1), np.uint32)
    w = np.zeros(max(e, 1), np.uint8) if weighted else None
    lib.ref_graph_transfer(h, rank if n else np.zeros(1, np.uint32), off, adj,
                           None if w is None else w.ctypes.data_as(C.c_void_p))
    from parallel_distance_oracle_gb300.graphs import CSRGraph
    return CSRGraph(n, off, adj[:e].copy(), None if w is None else w[:e].copy()), rank


def ref_graph_file(path, weighted: bool = False):
    """The reference reading an edge-list file (Graph(const char *),
    graph.h:95-117; weighted :262-290) and relabeling it (id_transfer)."""
    lib = ref(50)
    h = lib.ref_graph_read(str(path).encode(), int(weighted))
    try:
        return _ranked_from_ref(lib, h, weighted)
    finally:
        lib.ref_graph_free(h)


def ref_graph_edges(u, v, w=None):
    """The reference's Graph(edge_list) / WeightedGraph(edge_list, weights)
    (graph.h:125-153, :292-309) followed by id_transfer."""
    lib = ref(50)
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    wc = None if w is None else _c(w, np.uint8)
    h = lib.ref_graph_make(len(u), u, v, None if wc is None else wc.ctypes.data_as(C.c_void_p))
    try:
        return _ranked_from_ref(lib, h, w is not None)
    finally:
        lib.ref_graph_free(h)


def graph_ingest(u, v, w=None, n: int = 0, dedupe: bool = False):
    """The restatement of the same preparation (orc_graph_ingest); n = 0
    takes max id + 1.  Returns (CSRGraph, rank)."""
    from parallel_distance_oracle_gb300.graphs import CSRGraph
    lib = port()
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    m = len(u)
    if n == 0 and m:
        n = int(max(u.max(), v.max())) + 1
    wc = None if w is None else _c(w, np.uint8)
    off = np.zeros(n + 1, np.uint64)
    adj = np.zeros(max(2 * m, 1), np.uint32)
    wo = np.zeros(max(2 * m, 1), np.uint8) if w is not None else None
    rank = np.zeros(max(n, 1), np.uint32)
    ent, nn = C.c_uint64(), C.c_uint32()
    vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = lib.orc_graph_ingest(m, vp(u), vp(v), vp(wc), n, int(dedupe), off, adj, vp(wo), rank, C.byref(ent),
                              C.byref(nn))
    if rc != 0:
        raise ValueError("edge endpoint out of range")
    e = ent.value
    return CSRGraph(n, off, adj[:e].copy(), None if wo is None else wo[:e].copy()), rank[:n]


def parse_edge_text(text: bytes, weighted: bool = False):
    """orc_edge_text_parse: (u, v, w) from edge-list text; w None when unweighted."""
    lib = port()
    cnt = lib.orc_edge_text_parse(text, len(text), int(weighted), 0, None, None, None)
    u = np.zeros(max(cnt, 1), np.uint32)
    v = np.zeros(max(cnt, 1), np.uint32)
    w = np.zeros(max(cnt, 1), np.uint8) if weighted else None
    vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    lib.orc_edge_text_parse(text, len(text), int(weighted), cnt, vp(u), vp(v), vp(w))
    return u[:cnt].copy(), v[:cnt].copy(), None if w is None else w[:cnt].copy()


def ref_unw_label(g, rank, K: int, B: int, mode: int = 0, threads: int = 1) -> UnwLabels:
    lib = ref(K)
    lib.ref_set_threads(threads)
    h = lib.ref_unw_build(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(rank, np.uint32), B, mode)
    if not h:
        raise ValueError(f"reference driver has no batch size {B}")
    try:
        tot = lib.ref_unw_num_labels(h)
        off = np.zeros(g.n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.uint8)
        bpd = np.zeros(max(g.n * K, 1), np.uint8)
        bps = np.zeros(max(g.n * K * 2, 1), np.uint64)
        lib.ref_unw_export(h, off, hub, dist, bpd, bps)
        secs = lib.ref_unw_seconds(h)
    finally:
        lib.ref_unw_free(h)
    return UnwLabels(g.n, K, off, hub[:tot], dist[:tot], bpd[: g.n * K], bps[: g.n * K * 2], seconds=secs)


def ref_w_label(g, rank, B: int, mode: int = 0, threads: int = 1) -> WLabels:
    lib = ref(50)
    lib.ref_set_threads(threads)
    h = lib.ref_w_build(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(g.w, np.uint8),
                        _c(rank, np.uint32), B, mode)
    if not h:
        raise ValueError(f"reference driver has no batch size {B}")
    try:
        tot = lib.ref_w_num_labels(h)
        off = np.zeros(g.n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.int16)
        lib.ref_w_export(h, off, hub, dist)
        secs = lib.ref_w_seconds(h)
    finally:
        lib.ref_w_free(h)
    return WLabels(g.n, off, hub[:tot], dist[:tot], seconds=secs)


def ref_unw_store(g, rank, K: int, B: int, path) -> None:
    """The reference labels g (VertexCentricPLL<B>, K BP roots) and writes
    its index file with its own store_index_to_file."""
    lib = ref(K)
    if lib.ref_unw_store(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(rank, np.uint32), B,
                         str(path).encode()) != 0:
        raise ValueError(f"reference driver has no batch size {B}")


def ref_w_store(g, rank, B: int, path) -> None:
    """WeightedVertexCentricPLL<B> over g, then its store_index_to_file."""
    lib = ref(50)
    if lib.ref_w_store(g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(g.w, np.uint8), _c(rank, np.uint32), B,
                       str(path).encode()) != 0:
        raise ValueError(f"reference driver has no batch size {B}")


def ref_load_query(path, a, b, weighted: bool = False, K: int = 50) -> np.ndarray:
    """The reference's load_index_from_file on `path`, then its
    query_distance for every pair (query_distance.cpp's loop).  K must be the
    file's root count (unweighted)."""
    a, b = _c(a, np.uint32), _c(b, np.uint32)
    if weighted:
        out = np.zeros(len(a), np.int16)
        n = ref(50).ref_w_load_query(str(path).encode(), len(a), a, b, out)
    else:
        out = np.zeros(len(a), np.uint8)
        n = ref(K).ref_unw_load_query(str(path).encode(), len(a), a, b, out)
    if n < 0:
        raise ValueError(f"reference loader could not read {path} (missing, or another root count)")
    return out


_refvec = None


def refvec_available() -> bool:
    """The reference's AVX-512 labelers are built (x86 host with AVX-512)."""
    return _b.vec_so().exists() or _b.build_reference_vec() is not None


def refvec() -> C.CDLL:
    global _refvec
    if _refvec is None:
        so = _b.build_reference_vec()
        if so is None:
            raise FileNotFoundError("the reference's AVX-512 classes cannot be built on this host")
        lib = C.CDLL(str(so))
        lib.refvec_set_threads.argtypes = [C.c_int]
        lib.refvec_unw_build.restype = C.c_void_p
        lib.refvec_unw_build.argtypes = [C.c_uint32, _u64p, _u32p, _u32p, C.c_uint32, C.c_int]
        lib.refvec_w_build.restype = C.c_void_p
        lib.refvec_w_build.argtypes = [C.c_uint32, _u64p, _u32p, _u8p, _u32p, C.c_uint32, C.c_int]
        lib.refvec_num_labels.restype = C.c_uint64
        lib.refvec_num_labels.argtypes = [C.c_void_p]
        lib.refvec_export.argtypes = [C.c_void_p, _u64p, _u32p, _i16p, C.c_void_p, C.c_void_p]
        lib.refvec_free.argtypes = [C.c_void_p]
        _refvec = lib
    return _refvec


def refvec_label(g, rank, B: int, weighted: bool, mode: int = 0, threads: int = 1):
    """Canonical labels of the reference's AVX-512 class (mode 0 sequential,
    1 OpenMP; 50 BP roots unweighted).  UnwLabels or WLabels."""
    lib = refvec()
    lib.refvec_set_threads(threads)
    args = (g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32))
    if weighted:
        h = lib.refvec_w_build(*args, _c(g.w, np.uint8), _c(rank, np.uint32), B, mode)
    else:
        h = lib.refvec_unw_build(*args, _c(rank, np.uint32), B, mode)
    if not h:
        raise ValueError(f"no AVX-512 class instance for batch size {B}")
    try:
        tot = lib.refvec_num_labels(h)
        off = np.zeros(g.n + 1, np.uint64)
        hub = np.zeros(max(tot, 1), np.uint32)
        dist = np.zeros(max(tot, 1), np.int16)
        K = 0 if weighted else 50
        bpd = np.zeros(max(g.n * K, 1), np.uint8)
        bps = np.zeros(max(g.n * K * 2, 1), np.uint64)
        lib.refvec_export(h, off, hub, dist, bpd.ctypes.data_as(C.c_void_p), bps.ctypes.data_as(C.c_void_p))
    finally:
        lib.refvec_free(h)
    if weighted:
        return WLabels(g.n, off, hub[:tot], dist[:tot])
    return UnwLabels(g.n, K, off, hub[:tot], dist[:tot].astype(np.uint8), bpd[: g.n * K], bps[: g.n * K * 2])


def same_unw(a: UnwLabels, b: UnwLabels) -> bool:
    return (a.n == b.n and a.K == b.K and np.array_equal(a.off, b.off) and np.array_equal(a.hub, b.hub)
            and np.array_equal(a.dist, b.dist) and np.array_equal(a.bpd, b.bpd)
            and np.array_equal(a.bps, b.bps))


def same_w(a: WLabels, b: WLabels) -> bool:
    return (a.n == b.n and np.array_equal(a.off, b.off) and np.array_equal(a.hub, b.hub)
            and np.array_equal(a.dist.astype(np.int64), b.dist.astype(np.int64)))


def unw_prefix_sample(g, rank, K: int, B: int, nbatches: int, threads: int = 0):
    """Bounded CPU timing sample: BP labeling + the first ``nbatches`` batches.
    Uses the reference's ParaVertexCentricPLL when its driver is built on this
    host (kind "reference", all host threads), else the sequential
    restatement (kind "port", 1 thread).  Returns a dict."""
    import os
    labels = C.c_uint64(0)
    bp = C.c_double(0)
    args = (g.n, _c(g.off, np.uint64), _c(g.adj, np.uint32), _c(rank, np.uint32))
    if ref_available(K):
        lib = ref(K)
        t = threads or os.cpu_count() or 1
        lib.ref_set_threads(t)
        secs = lib.ref_unw_prefix(*args, B, nbatches, C.byref(labels), C.byref(bp))
        kind, cores = "reference", t
    else:
        secs = port().orc_unw_prefix(*args, K, B, nbatches, C.byref(labels), C.byref(bp))
        kind, cores = "port", 1
    return {"seconds": secs, "labels": int(labels.value), "bp_seconds": bp.value, "kind": kind, "cores": cores}


# ---- graph reductions --------------------------------------------------------

def _edges_n(u, v, n):
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    if n == 0 and len(u):
        n = int(max(u.max(), v.max())) + 1
    return u, v, n


def reduce_degree1(u, v, n: int = 0):
    """orc_reduce_degree1 (the reference's degree-1 chain deletion).  n = 0
    takes max id + 1.  Returns (deleted uint8[n], kept edge indices,
    nonterminating)."""
    u, v, n = _edges_n(u, v, n)
    m = len(u)
    deleted = np.zeros(max(n, 1), np.uint8)
    kept = np.zeros(max(m, 1), np.uint64)
    k, nt = C.c_uint64(), C.c_int()
    if port().orc_reduce_degree1(m, u, v, n, deleted, kept, C.byref(k), C.byref(nt)) != 0:
        raise ValueError("edge endpoint out of range")
    return deleted[:n], kept[:k.value].copy(), bool(nt.value)


def reduce_equivalent(u, v, n: int = 0):
    """orc_reduce_equivalent (the reference's equivalent-vertex removal).
    Returns (redundant uint8[n], new_id uint32[n], kept edge indices, n_out)."""
    u, v, n = _edges_n(u, v, n)
    m = len(u)
    red = np.zeros(max(n, 1), np.uint8)
    nid = np.zeros(max(n, 1), np.uint32)
    kept = np.zeros(max(m, 1), np.uint64)
    k, nout = C.c_uint64(), C.c_uint32()
    if port().orc_reduce_equivalent(m, u, v, n, red, nid, kept, C.byref(k), C.byref(nout)) != 0:
        raise ValueError("edge endpoint out of range")
    return red[:n], nid[:n], kept[:k.value].copy(), int(nout.value)


def ref_tools_available() -> bool:
    from oracle import build_oracle
    return all(build_oracle.ref_tool(t).exists() for t in build_oracle.REF_TOOLS)


def _write_edges(path, u, v):
    with open(path, "w") as f:
        f.write("".join(f"{a} {b}\n" for a, b in zip(u.tolist(), v.tolist())))


def ref_delete_degree1(u, v, timeout: float = 60.0) -> np.ndarray:
    """The reference's delete_1-degree tool on the edge list: its output
    edges, shape (k, 2), in the order it writes them."""
    import subprocess
    import tempfile
    from oracle import build_oracle
    with tempfile.TemporaryDirectory() as d:
        fin, fout = f"{d}/in.txt", f"{d}/out.txt"
        _write_edges(fin, _c(u, np.uint32), _c(v, np.uint32))
        subprocess.run([str(build_oracle.ref_tool("delete_1_degree")), fin, fout], check=True, timeout=timeout,
                       stdout=subprocess.DEVNULL)
        rows = [ln.split() for ln in open(fout).read().splitlines() if ln.strip()]
    return np.array(rows, np.uint32).reshape(-1, 2)


def ref_remove_equivalent(u, v, timeout: float = 60.0):
    """The reference's remove_equivalent_vertices tool: (num_v, edges (k, 2))
    read from the binary file it writes."""
    import subprocess
    import tempfile
    from oracle import build_oracle
    with tempfile.TemporaryDirectory() as d:
        fin, fout, flog = f"{d}/in.txt", f"{d}/out.bin", f"{d}/log.txt"
        _write_edges(fin, _c(u, np.uint32), _c(v, np.uint32))
        open(flog, "w").close()
        subprocess.run([str(build_oracle.ref_tool("remove_equivalent")), fin, fout, flog], check=True,
                       timeout=timeout, stdout=subprocess.DEVNULL, env={"OMP_NUM_THREADS": "1"})
        b = open(fout, "rb").read()
    nv = int(np.frombuffer(b[:4], np.uint32)[0])
    ne = int(np.frombuffer(b[4:12], np.uint64)[0])
    return nv, np.frombuffer(b[12:12 + 8 * ne], np.uint32).reshape(-1, 2).copy()
