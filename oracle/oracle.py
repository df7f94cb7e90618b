"""ctypes binding of the CPU oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

The oracle restates the reference's CPU BFS paths (crates/cpu_bfs) and graph
helpers (crates/core/src/graph.rs). Only the tests, the smoke check and the
benchmark's CPU-baseline leg use it, as the checker; the engine never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
u32p = C.POINTER(C.c_uint32)
UNREACHABLE = 0xFFFFFFFF

_lib = None


def build() -> Path:
    import platform
    stamp = HERE / "_build" / "arch.txt"
    arch = platform.machine()
    force = not stamp.exists() or stamp.read_text().strip() != arch
    subprocess.run(["make", "-s", "-C", str(HERE)] + (["-B"] if force else []), check=True)
    stamp.write_text(arch + "\n")
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        h = C.CDLL(str(LIB))
        h.oracle_ms_bfs_fifo.argtypes = [C.c_size_t, u32p, u32p, u32p, C.c_size_t, u32p,
                                         C.POINTER(C.c_size_t)]
        h.oracle_ms_bfs_threaded.argtypes = [C.c_size_t, u32p, u32p, u32p, C.c_size_t, u32p,
                                             C.c_int, C.POINTER(C.c_size_t)]
        h.oracle_ms_bfs_bit_parallel.argtypes = [C.c_size_t, u32p, u32p, u32p, C.c_size_t,
                                                 u32p, C.POINTER(C.c_size_t)]
        h.oracle_reachability_from_distances.argtypes = [C.c_size_t, C.c_size_t, u32p, u32p]
        h.oracle_reachability_from_distances.restype = None
        h.oracle_traversed_edges.argtypes = [C.c_size_t, u32p, C.c_size_t, u32p]
        h.oracle_traversed_edges.restype = C.c_uint64
        h.oracle_csr_from_edge_list.argtypes = [C.c_size_t, C.c_size_t, u32p, u32p, u32p, u32p,
                                                C.POINTER(C.c_size_t)]
        h.oracle_csr_from_edge_list.restype = None
        h.oracle_to_csc.argtypes = [C.c_size_t, C.c_size_t, u32p, u32p, u32p, u32p]
        h.oracle_to_csc.restype = None
        h.oracle_is_symmetric.argtypes = [C.c_size_t, C.c_size_t, u32p, u32p]
        _lib = h
    return _lib


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _p(a: np.ndarray):
    return a.ctypes.data_as(u32p)


class SourceOutOfBounds(ValueError):
    def __init__(self, source: int, index: int, V: int):
        super().__init__(f"Source vertex {source} at index {index} exceeds graph vertex "
                         f"count {V}")
        self.index = index


def _run(fn, V, row_offsets, col_indices, sources, *extra) -> np.ndarray:
    ro, ci, src = _u32(row_offsets), _u32(col_indices), _u32(sources)
    if ci.size == 0:
        ci = np.zeros(1, np.uint32)
    S = src.size
    if S == 0 or V == 0:
        return np.zeros(0, np.uint32)
    out = np.empty(S * V, np.uint32)
    bad = C.c_size_t(0)
    rc = fn(V, _p(ro), _p(ci), _p(src), S, _p(out), *extra, C.byref(bad))
    if rc == 1:
        raise SourceOutOfBounds(int(src[bad.value]), bad.value, V)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out


def ms_bfs_fifo(V, row_offsets, col_indices, sources) -> np.ndarray:
    """crates/cpu_bfs/src/fifo.rs:70-102."""
    return _run(lib().oracle_ms_bfs_fifo, V, row_offsets, col_indices, sources)


def ms_bfs_threaded(V, row_offsets, col_indices, sources, threads: int = 0) -> np.ndarray:
    """crates/cpu_bfs/src/rayon_ms.rs:11-54 (threads=0: all online cores)."""
    return _run(lib().oracle_ms_bfs_threaded, V, row_offsets, col_indices, sources,
                C.c_int(threads))


def ms_bfs_bit_parallel(V, row_offsets, col_indices, sources) -> np.ndarray:
    """crates/cpu_bfs/src/bit_parallel.rs:101-130."""
    return _run(lib().oracle_ms_bfs_bit_parallel, V, row_offsets, col_indices, sources)


def reachability_from_distances(V: int, S: int, dist) -> np.ndarray:
    """crates/core/src/graph.rs:571-646."""
    wpv = (S + 31) // 32
    out = np.zeros(V * wpv, np.uint32)
    if S and V:
        d = _u32(dist)
        lib().oracle_reachability_from_distances(V, S, _p(d), _p(out))
    return out


def traversed_edges(V: int, row_offsets, S: int, dist) -> int:
    """crates/cli/src/bench.rs:478-491."""
    return int(lib().oracle_traversed_edges(V, _p(_u32(row_offsets)), S, _p(_u32(dist))))


def csr_from_edge_list(V: int, edges):
    """crates/core/src/graph.rs:51-79 -> (row_offsets, col_indices)."""
    e = np.asarray(edges, dtype=np.uint32).reshape(-1, 2)
    u, v = _u32(e[:, 0]), _u32(e[:, 1])
    ro = np.zeros(V + 1, np.uint32)
    ci = np.zeros(max(1, len(e)), np.uint32)
    n = C.c_size_t(0)
    lib().oracle_csr_from_edge_list(V, len(e), _p(u) if len(e) else None,
                                    _p(v) if len(e) else None, _p(ro), _p(ci), C.byref(n))
    return ro, ci[:n.value].copy()


def to_csc(V: int, row_offsets, col_indices):
    """crates/core/src/graph.rs:90-127 -> (col_offsets, row_indices)."""
    ro, ci = _u32(row_offsets), _u32(col_indices)
    E = ci.size
    co = np.zeros(V + 1, np.uint32)
    ri = np.zeros(max(1, E), np.uint32)
    lib().oracle_to_csc(V, E, _p(ro), _p(ci if E else np.zeros(1, np.uint32)), _p(co), _p(ri))
    return co, ri[:E].copy()


def is_symmetric(V: int, row_offsets, col_indices) -> bool:
    """crates/core/src/graph.rs:129-133."""
    ro, ci = _u32(row_offsets), _u32(col_indices)
    E = ci.size
    return bool(lib().oracle_is_symmetric(V, E, _p(ro), _p(ci if E else np.zeros(1, np.uint32))))
