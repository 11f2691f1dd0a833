"""ctypes binding of include/pado_gpu.h (libpado_gpu.so, built in-tree).

There is no CPU fallback: if the CUDA library is missing or fails to load,
importing this module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

PADO_OK = 0
PADO_UNWEIGHTED = 0
PADO_WEIGHTED = 1
PADO_INGEST_DEDUPE = 1


class PadoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class Info(C.Structure):
    _fields_ = [("n", C.c_uint32), ("kind", C.c_uint32), ("bp_roots", C.c_uint32), ("batch", C.c_uint32),
                ("num_labels", C.c_uint64), ("build_seconds", C.c_double), ("bp_seconds", C.c_double),
                ("device_bytes", C.c_uint64), ("levels", C.c_uint32), ("batches", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("batches", C.c_uint64), ("pairs", C.c_uint64),
                ("max_batch_pairs", C.c_uint64), ("admissions", C.c_uint64), ("evictions", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("resident_indexes", C.c_uint32), ("pad", C.c_uint32)]


def _load() -> C.CDLL:
    lib_path: Path = _build.LIB
    if not _build.up_to_date():
        try:
            _build.build()
        except Exception as e:  # no toolchain: a stale library is still usable
            if not lib_path.exists():
                raise ImportError(f"libpado_gpu.so is not built and cannot be built: {e}") from e
    lib = C.CDLL(str(lib_path))
    vp = C.c_void_p
    u32, u64 = C.c_uint32, C.c_uint64
    P = C.POINTER
    sig = {
        "pado_last_error": (C.c_char_p, []),
        "pado_status_string": (C.c_char_p, [C.c_int]),
        "pado_version": (C.c_char_p, []),
        "pado_unw_build": (C.c_int, [u32, vp, vp, vp, u32, u32, P(vp)]),
        "pado_unw_build_ranked": (C.c_int, [u32, vp, vp, u32, u32, P(vp)]),
        "pado_unw_build_many": (C.c_int, [u32, vp, vp, vp, vp, u32, u32, vp]),
        "pado_unw_tune_batch": (C.c_int, [u32, vp, vp, vp, vp, u32, vp, u32, u32, P(u32), vp]),
        "pado_w_build": (C.c_int, [u32, vp, vp, vp, vp, u32, P(vp)]),
        "pado_w_build_ranked": (C.c_int, [u32, vp, vp, vp, u32, P(vp)]),
        "pado_graph_ingest": (C.c_int, [u64, vp, vp, vp, u32, u32, vp, vp, vp, vp, P(u64)]),
        "pado_graph_ingest_device": (C.c_int, [u64, vp, vp, vp, u32, u32, vp, vp, vp, vp, P(u64), vp]),
        "pado_set_scratch_cache": (C.c_int, [u64]),
        "pado_reduce_degree1": (C.c_int, [u64, vp, vp, u32, vp, vp, P(u64)]),
        "pado_reduce_equivalent": (C.c_int, [u64, vp, vp, u32, vp, vp, vp, P(u64), P(u32)]),
        "pado_reduce_degree1_device": (C.c_int, [u64, vp, vp, u32, vp, vp, P(u64), vp]),
        "pado_reduce_equivalent_device": (C.c_int, [u64, vp, vp, u32, vp, vp, vp, P(u64), P(u32), vp]),
        "pado_unw_build_edges": (C.c_int, [u64, vp, vp, u32, u32, u32, u32, P(vp)]),
        "pado_w_build_edges": (C.c_int, [u64, vp, vp, vp, u32, u32, u32, P(vp)]),
        "pado_build_edge_file": (C.c_int, [C.c_char_p, u32, u32, u32, u32, P(vp)]),
        "pado_edge_text_parse": (C.c_int, [vp, u64, u32, u64, vp, vp, vp, P(u64)]),
        "pado_set_order": (C.c_int, [vp, vp]),
        "pado_free": (None, [vp]),
        "pado_get_info": (C.c_int, [vp, P(Info)]),
        "pado_export": (C.c_int, [vp, vp, vp, vp, vp, vp]),
        "pado_import": (C.c_int, [u32, u32, u32, vp, vp, vp, vp, vp, P(vp)]),
        "pado_query": (C.c_int, [vp, u64, vp, vp, vp]),
        "pado_query_device": (C.c_int, [vp, u64, vp, vp, vp, vp]),
        "pado_store": (C.c_int, [vp, C.c_char_p]),
        "pado_load": (C.c_int, [C.c_char_p, u32, P(vp)]),
        "pado_query_noalloc": (C.c_int, [vp, u64, vp, vp, vp]),
        "pado_kernel_launches": (u64, []),
        "pado_debug_fail_alloc": (C.c_int, [u64]),
        "pado_debug_live_allocations": (C.c_int64, []),
        "pado_selftest_barrier": (C.c_int, [u32, u32, u64, P(u32)]),
        "pado_server_create": (C.c_int, [u64, u32, u32, P(vp)]),
        "pado_server_add": (C.c_int, [vp, vp, P(u32)]),
        "pado_server_submit": (C.c_int, [vp, u32, u64, vp, vp, vp, P(u64)]),
        "pado_server_wait": (C.c_int, [vp, u64, C.c_double, P(C.c_double)]),
        "pado_server_get_stats": (C.c_int, [vp, P(ServerStats)]),
        "pado_server_replay": (C.c_int, [vp, u64, vp, vp, vp, vp, vp, vp, vp, vp, u32, vp]),
        "pado_server_destroy": (None, [vp]),
        "pado_profile": (C.c_int, [C.c_int]),
        "pado_profile_read": (C.c_size_t, [C.c_char_p, C.c_size_t, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()

# Every symbol include/pado_gpu.h declares (checked by the CPU test suite).
EXPORTED = [
    "pado_last_error", "pado_status_string", "pado_version", "pado_unw_build", "pado_unw_build_ranked",
    "pado_unw_build_many", "pado_unw_tune_batch",
    "pado_w_build", "pado_w_build_ranked", "pado_graph_ingest", "pado_graph_ingest_device",
    "pado_set_scratch_cache", "pado_reduce_degree1", "pado_reduce_equivalent", "pado_reduce_degree1_device",
    "pado_reduce_equivalent_device",
    "pado_unw_build_edges", "pado_w_build_edges",
    "pado_build_edge_file", "pado_edge_text_parse", "pado_set_order", "pado_free", "pado_get_info", "pado_export",
    "pado_import", "pado_query", "pado_query_device", "pado_query_noalloc", "pado_store", "pado_load",
    "pado_kernel_launches", "pado_debug_fail_alloc", "pado_debug_live_allocations", "pado_selftest_barrier",
    "pado_server_create", "pado_server_add", "pado_server_submit", "pado_server_wait",
    "pado_server_get_stats", "pado_server_replay", "pado_server_destroy",
    "pado_profile", "pado_profile_read",
]


def check(status: int) -> None:
    if status != PADO_OK:
        raise PadoError(status, lib.pado_last_error().decode(errors="replace"))


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
