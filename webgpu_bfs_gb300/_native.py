"""ctypes binding of include/msbfs.h (libmsbfs.so).

The shared library is built in-tree by webgpu_bfs_gb300/build.py. There is no
fallback: if the library is missing or does not export the declared symbols,
loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libmsbfs.so"

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
sizep = C.POINTER(C.c_size_t)


class Stats(C.Structure):
    _fields_ = [
        ("method", C.c_uint32),
        ("path", C.c_uint32),
        ("passes", C.c_uint32),
        ("words_per_vertex", C.c_uint32),
        ("levels", C.c_uint32),
        ("push_levels", C.c_uint32),
        ("pull_levels", C.c_uint32),
        ("cta_cluster", C.c_uint32),
        ("reached_pairs", C.c_uint64),
        ("gpu_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class LevelRecord(C.Structure):
    _fields_ = [
        ("pass_", C.c_uint32),
        ("level", C.c_uint32),
        ("dir", C.c_uint32),
        ("frontier_vertices", C.c_uint32),
        ("frontier_entries", C.c_uint64),
        ("active", C.c_uint64),
        ("edges", C.c_uint64),
        ("new_vertices", C.c_uint64),
        ("new_pairs", C.c_uint64),
        ("rows", C.c_uint64),
        ("device_ms", C.c_double),
        ("event_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["pass"] = d.pop("pass_")
        return d


class Csr(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_size_t),
        ("num_edges", C.c_size_t),
        ("row_offsets", u32p),
        ("col_indices", u32p),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("slots", C.c_uint32),
        ("max_sources_per_launch", C.c_uint32),
        ("hbm_budget_bytes", C.c_uint64),
        ("method", C.c_int),
        ("express_slots", C.c_uint32),
        ("small_sources", C.c_uint32),
        ("general_sm_percent", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class RequestInfo(C.Structure):
    _fields_ = [
        ("latency_ms", C.c_double),
        ("queue_ms", C.c_double),
        ("launches", C.c_uint32),
        ("status", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class MtxErrorInfo(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("line_number", C.c_uint64),
        ("row", C.c_uint64),
        ("col", C.c_uint64),
        ("max_rows", C.c_uint64),
        ("max_cols", C.c_uint64),
        ("message", C.c_char * 256),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("max_words_per_pass", C.c_uint32),
        ("alpha", C.c_uint32),
        ("beta", C.c_uint32),
        ("hub_split", C.c_uint32),
        ("bitmap_div", C.c_uint32),
        ("warp_scan_degree", C.c_uint32),
        ("from_cache", C.c_uint32),
        ("trials", C.c_uint32),
        ("level_path", C.c_uint32),
        ("ms", C.c_double),
        ("default_ms", C.c_double),
        ("class_name", C.c_char * 48),
    ]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["class_name"] = d["class_name"].decode()
        return d


# numpy view of msbfs_source_stats
SOURCE_STATS_DTYPE = [("distance_sum", "<u8"), ("eccentricity", "<u4"), ("reached", "<u4")]


class BatchGraph(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_size_t),
        ("num_edges", C.c_size_t),
        ("row_offsets", u32p),
        ("col_indices", u32p),
        ("sources", u32p),
        ("num_sources", C.c_size_t),
    ]


# name -> (restype, argtypes); every function declared in include/msbfs.h.
SIGNATURES = {
    "msbfs_engine_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "msbfs_engine_destroy": (None, [C.c_void_p]),
    "msbfs_engine_method": (C.c_int, [C.c_void_p]),
    "msbfs_engine_last_error": (C.c_char_p, [C.c_void_p]),
    "msbfs_engine_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "msbfs_engine_set_tuning": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]),
    "msbfs_engine_set_sm_share": (C.c_int, [C.c_void_p, C.c_uint32]),
    "msbfs_engine_autotune": (C.c_int, [C.c_void_p, C.c_void_p, u32p, C.c_size_t, C.c_char_p,
                                        C.POINTER(Tuning)]),
    "msbfs_engine_set_level_cap": (C.c_int, [C.c_void_p, C.c_uint32]),
    "msbfs_engine_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "msbfs_engine_level_log": (C.c_int, [C.c_void_p, C.POINTER(LevelRecord), C.c_size_t,
                                         sizep]),
    "msbfs_select_auto_method": (C.c_int, [C.c_size_t, C.c_size_t, u32p, C.c_size_t]),
    "msbfs_graph_create": (C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, u32p, u32p,
                                     C.POINTER(C.c_void_p)]),
    "msbfs_graph_destroy": (None, [C.c_void_p]),
    "msbfs_graph_info": (C.c_int, [C.c_void_p, sizep, sizep, u32p, C.POINTER(C.c_int)]),
    "msbfs_run_ms_bfs": (C.c_int, [C.c_void_p, C.c_void_p, u32p, C.c_size_t, u32p,
                                   C.POINTER(Stats)]),
    "msbfs_run_ms_bfs_with_method": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, u32p,
                                               C.c_size_t, u32p, C.POINTER(Stats)]),
    "msbfs_run_ms_bfs_csr": (C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, u32p, u32p, u32p,
                                       C.c_size_t, u32p, C.POINTER(Stats)]),
    "msbfs_run_ms_bfs_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, u32p, C.c_size_t,
                                          C.c_void_p]),
    "msbfs_engine_synchronize": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "msbfs_run_reachability": (C.c_int, [C.c_void_p, C.c_void_p, u32p, C.c_size_t, u32p,
                                         C.POINTER(Stats)]),
    "msbfs_traversed_edges_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                               u64p]),
    "msbfs_run_cta_noalloc": (C.c_int, [C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, u32p,
                                        C.c_size_t, C.c_void_p, C.c_void_p]),
    "msbfs_run_ms_bfs_stats_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, u32p,
                                                C.c_size_t, C.c_void_p]),
    "msbfs_run_ms_bfs_stats": (C.c_int, [C.c_void_p, C.c_void_p, u32p, C.c_size_t, C.c_void_p,
                                         C.POINTER(Stats)]),
    "msbfs_server_create": (C.c_int, [C.c_int, C.c_size_t, C.c_size_t, u32p, u32p,
                                      C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "msbfs_server_submit": (C.c_int, [C.c_void_p, u32p, C.c_size_t, C.c_int, C.c_void_p,
                                      C.POINTER(C.c_uint64)]),
    "msbfs_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double,
                                    C.POINTER(RequestInfo)]),
    "msbfs_server_counters": (C.c_int, [C.c_void_p, u64p, u64p]),
    "msbfs_server_destroy": (None, [C.c_void_p]),
    "msbfs_batch_create": (C.c_int, [C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "msbfs_batch_destroy": (None, [C.c_void_p]),
    "msbfs_batch_autotune": (C.c_int, [C.c_void_p, C.c_size_t, C.c_char_p]),
    "msbfs_batch_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "msbfs_batch_run_per_graph": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "msbfs_batch_result": (C.c_int, [C.c_void_p, C.c_size_t, u32p]),
    "msbfs_batch_config": (C.c_int, [C.c_void_p, C.c_size_t, u32p, u32p, u32p, C.c_char_p,
                                     C.c_size_t]),
    "msbfs_csr_free": (None, [C.POINTER(Csr)]),
    "msbfs_csr_from_edge_list": (C.c_int, [C.c_size_t, C.c_size_t, u32p, u32p,
                                           C.POINTER(Csr)]),
    "msbfs_csr_transpose": (C.c_int, [C.POINTER(Csr), C.POINTER(Csr)]),
    "msbfs_csr_is_symmetric": (C.c_int, [C.POINTER(Csr)]),
    "msbfs_csr_to_undirected": (C.c_int, [C.POINTER(Csr), C.POINTER(Csr)]),
    "msbfs_csr_validate": (C.c_int, [C.POINTER(Csr), C.c_char_p, C.c_size_t]),
    "msbfs_csr_max_degree": (C.c_uint32, [C.POINTER(Csr)]),
    "msbfs_mtx_parse": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(Csr),
                                  C.POINTER(MtxErrorInfo)]),
    "msbfs_mtx_read": (C.c_int, [C.c_char_p, C.POINTER(Csr), C.POINTER(MtxErrorInfo)]),
    "msbfs_gen_grid2d": (C.c_int, [C.c_size_t, C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_erdos_renyi_np": (C.c_int, [C.c_size_t, C.c_double, C.c_uint64,
                                           C.POINTER(Csr)]),
    "msbfs_gen_random_tree": (C.c_int, [C.c_size_t, C.c_uint64, C.POINTER(Csr)]),
    "msbfs_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_uint64, C.c_int, C.POINTER(Csr)]),
    "msbfs_gen_path": (C.c_int, [C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_star": (C.c_int, [C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_cycle": (C.c_int, [C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_clique": (C.c_int, [C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_disconnected_cliques": (C.c_int, [sizep, C.c_size_t, C.POINTER(Csr)]),
    "msbfs_gen_wilson_grid": (C.c_int, [C.c_size_t, C.c_size_t, C.c_size_t, C.c_uint64,
                                        C.POINTER(Csr)]),
    "msbfs_sample_sources": (C.c_int, [C.POINTER(Csr), C.c_size_t, C.c_uint64, C.c_uint32,
                                       u32p]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Loads libmsbfs.so once and binds every declared entry point."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = os.environ.get("MSBFS_LIB", str(LIB_PATH))
        if not Path(path).exists():
            raise ImportError(
                f"libmsbfs.so not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        handle = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)  # AttributeError if a symbol is missing
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib
