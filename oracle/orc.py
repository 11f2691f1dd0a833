"""ctypes wrappers over the oracle (liboracle.so) and the reference driver
(oracle/_ref/libpado_ref_k*.so).  TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

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
             "bp_pruned", "dist_checks", "dist_entries", "labels_added", "root_rows"]
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
        _refs[K] = lib
    return _refs[K]


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
