"""GB300-native multi-source BFS engine (host mirror of the reference API).

Python mirror of the reference's public multi-source BFS surface, over the C
ABI of include/msbfs.h:

* ``CsrGraph`` / ``CscGraph`` / ``ReachabilityBitmask`` -- crates/core/src/graph.rs
* ``BfsEngine.run_ms_bfs`` -- crates/core/src/lib.rs:21-39
* ``GpuBfsMethod`` / ``GpuBfsEngine`` -- crates/gpu_bfs/src/engine.rs:33-490
* generators -- crates/core/src/generators.rs

All compute runs in libmsbfs.so (sm_103a CUDA kernels + C++ runtime); this
module only marshals numpy arrays. Errors are raised as ``BfsError`` with the
reference's messages (e.g. "Source vertex 7 at index 2 exceeds graph vertex
count 5").
"""
from __future__ import annotations

import ctypes as C
import enum
import threading
import weakref
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _native
from ._native import Csr, Stats, u32p

__all__ = [
    "BfsError", "CsrGraph", "CscGraph", "ReachabilityBitmask", "GpuBfsMethod",
    "GpuBfsEngine", "Grid2D", "generate_grid2d", "generate_erdos_renyi_np",
    "generate_random_tree", "generate_rmat", "generate_graph500_rmat", "empty_graph",
    "isolated_vertices", "single_vertex", "path_graph", "star_graph", "cycle_graph",
    "clique_graph", "disconnected_cliques", "wilson_grid", "sample_sources",
    "GRAPH500_A", "GRAPH500_B", "GRAPH500_C", "GRAPH500_D", "BfsServer", "BatchedBfs",
    "MtxError", "parse_mtx", "read_mtx", "SOURCE_STATS_DTYPE",
]

UNREACHABLE = 0xFFFFFFFF

ERROR_NAMES = {
    1: "SourceOutOfBounds", 2: "EmptyGraph", 3: "OutOfMemory", 4: "Timeout", 5: "Cuda",
    6: "InvalidGraph", 7: "InvalidArgument", 8: "NoDevice", 9: "ScratchTooSmall",
    10: "Parse",
}


class BfsError(RuntimeError):
    """Error returned by the engine; ``code`` is the MSBFS_ERR_* value."""

    def __init__(self, code: int, message: str):
        super().__init__(message or ERROR_NAMES.get(code, f"error {code}"))
        self.code = code


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(u32p)


def _take_csr(c: Csr):
    """Copies a library-allocated msbfs_csr into numpy arrays and frees it."""
    V, E = c.num_vertices, c.num_edges
    off = np.ctypeslib.as_array(c.row_offsets, shape=(V + 1,)).copy()
    idx = (np.ctypeslib.as_array(c.col_indices, shape=(E,)).copy() if E
           else np.zeros(0, np.uint32))
    _native.lib().msbfs_csr_free(C.byref(c))
    return V, E, off, idx


def _check(rc: int, msg: str = ""):
    if rc != 0:
        raise BfsError(rc, msg)


class CsrGraph:
    """Compressed Sparse Row graph (crates/core/src/graph.rs:8-22).

    ``row_offsets`` (V+1) and ``col_indices`` (E) are read-only u32 arrays;
    rows are sorted and free of duplicates and self-loops when built through
    ``from_edge_list`` or a generator.
    """

    __slots__ = ("num_vertices", "num_edges", "row_offsets", "col_indices", "__weakref__")

    def __init__(self, num_vertices: int, row_offsets, col_indices):
        self.num_vertices = int(num_vertices)
        self.row_offsets = _u32(row_offsets)
        self.col_indices = _u32(col_indices)
        self.num_edges = int(self.col_indices.size)
        self.row_offsets.flags.writeable = False
        self.col_indices.flags.writeable = False

    # -- construction ---------------------------------------------------------
    @classmethod
    def from_edge_list(cls, num_vertices: int, edges: Iterable[Sequence[int]]) -> "CsrGraph":
        """CsrGraph::from_edge_list (graph.rs:51-79)."""
        e = np.asarray(list(edges) if not isinstance(edges, np.ndarray) else edges,
                       dtype=np.int64).reshape(-1, 2)
        keep = (e[:, 0] >= 0) & (e[:, 1] >= 0) & (e[:, 0] < 2**32) & (e[:, 1] < 2**32)
        e = e[keep]
        u, v = _u32(e[:, 0]), _u32(e[:, 1])
        c = Csr()
        _check(_native.lib().msbfs_csr_from_edge_list(num_vertices, u.size, _ptr(u), _ptr(v),
                                                      C.byref(c)))
        V, _, off, idx = _take_csr(c)
        return cls(V, off, idx)

    def _as_csr(self) -> Csr:
        c = Csr()
        c.num_vertices = self.num_vertices
        c.num_edges = self.num_edges
        c.row_offsets = _ptr(self.row_offsets)
        c.col_indices = _ptr(self.col_indices)
        return c

    # -- structure ------------------------------------------------------------
    def to_csc(self) -> "CscGraph":
        """CsrGraph::to_csc (graph.rs:90-127)."""
        out = Csr()
        _check(_native.lib().msbfs_csr_transpose(C.byref(self._as_csr()), C.byref(out)))
        V, _, off, idx = _take_csr(out)
        return CscGraph(V, off, idx)

    def is_symmetric(self) -> bool:
        """CsrGraph::is_symmetric (graph.rs:129-133)."""
        return bool(_native.lib().msbfs_csr_is_symmetric(C.byref(self._as_csr())))

    def to_undirected(self) -> "CsrGraph":
        """CsrGraph::to_undirected (graph.rs:136-151)."""
        out = Csr()
        _check(_native.lib().msbfs_csr_to_undirected(C.byref(self._as_csr()), C.byref(out)))
        V, _, off, idx = _take_csr(out)
        return CsrGraph(V, off, idx)

    def validate(self) -> None:
        """CsrGraph::validate (graph.rs:226-280); raises BfsError when invalid."""
        buf = C.create_string_buffer(256)
        if self.row_offsets.size != self.num_vertices + 1:
            raise BfsError(6, f"row_offsets length {self.row_offsets.size} != "
                              f"{self.num_vertices + 1}")
        rc = _native.lib().msbfs_csr_validate(C.byref(self._as_csr()), buf, 256)
        _check(rc, buf.value.decode())

    def is_empty(self) -> bool:
        return self.num_vertices == 0

    def degree(self, u: int) -> int:
        if not 0 <= u < self.num_vertices:
            raise IndexError(f"Vertex {u} out of bounds for graph with "
                             f"{self.num_vertices} vertices")
        return int(self.row_offsets[u + 1] - self.row_offsets[u])

    def neighbors(self, u: int) -> np.ndarray:
        self.degree(u)
        return self.col_indices[self.row_offsets[u]:self.row_offsets[u + 1]]

    def degrees(self) -> np.ndarray:
        return np.diff(self.row_offsets.astype(np.int64))

    def max_degree(self) -> int:
        """CsrGraph::max_degree (graph.rs:209-214)."""
        return int(self.degrees().max()) if self.num_vertices else 0

    def avg_degree(self) -> float:
        return self.num_edges / self.num_vertices if self.num_vertices else 0.0

    def __eq__(self, other) -> bool:
        return (isinstance(other, CsrGraph) and self.num_vertices == other.num_vertices
                and np.array_equal(self.row_offsets, other.row_offsets)
                and np.array_equal(self.col_indices, other.col_indices))

    def __repr__(self) -> str:
        return f"CsrGraph(V={self.num_vertices}, E={self.num_edges})"


class CscGraph:
    """Compressed Sparse Column graph (crates/core/src/graph.rs:27-41)."""

    __slots__ = ("num_vertices", "num_edges", "col_offsets", "row_indices")

    def __init__(self, num_vertices: int, col_offsets, row_indices):
        self.num_vertices = int(num_vertices)
        self.col_offsets = _u32(col_offsets)
        self.row_indices = _u32(row_indices)
        self.num_edges = int(self.row_indices.size)

    def to_csr(self) -> CsrGraph:
        """CscGraph::to_csr (graph.rs:283-316): the same transpose."""
        return CsrGraph(self.num_vertices, self.col_offsets, self.row_indices).to_csc_as_csr()

    def in_degree(self, v: int) -> int:
        return int(self.col_offsets[v + 1] - self.col_offsets[v])

    def predecessors(self, v: int) -> np.ndarray:
        return self.row_indices[self.col_offsets[v]:self.col_offsets[v + 1]]

    def max_in_degree(self) -> int:
        return int(np.diff(self.col_offsets.astype(np.int64)).max()) if self.num_vertices else 0

    def validate(self) -> None:
        CsrGraph(self.num_vertices, self.col_offsets, self.row_indices).validate()


def _csr_to_csc_as_csr(self: CsrGraph) -> CsrGraph:
    csc = self.to_csc()
    return CsrGraph(csc.num_vertices, csc.col_offsets, csc.row_indices)


CsrGraph.to_csc_as_csr = _csr_to_csc_as_csr


class ReachabilityBitmask:
    """Vertex-major reachability bits (crates/core/src/graph.rs:446-646):
    ``words[v * words_per_vertex + s // 32] >> (s % 32) & 1``."""

    def __init__(self, num_vertices: int, num_sources: int, words=None):
        self.num_vertices = int(num_vertices)
        self.num_sources = int(num_sources)
        self.words_per_vertex = 0 if num_sources == 0 else (num_sources + 31) // 32
        n = self.num_vertices * self.words_per_vertex
        self.words = np.zeros(n, np.uint32) if words is None else _u32(words)
        if self.words.size != n:
            raise ValueError("Words buffer length must exactly equal "
                             "num_vertices * words_per_vertex")

    @classmethod
    def zeroed(cls, num_vertices: int, num_sources: int) -> "ReachabilityBitmask":
        return cls(num_vertices, num_sources)

    def is_reachable(self, s: int, v: int) -> bool:
        if s >= self.num_sources or v >= self.num_vertices or self.words_per_vertex == 0:
            return False
        w = self.words[v * self.words_per_vertex + s // 32]
        return bool((int(w) >> (s % 32)) & 1)

    def set_reachable(self, s: int, v: int) -> None:
        if s < self.num_sources and v < self.num_vertices and self.words_per_vertex:
            self.words[v * self.words_per_vertex + s // 32] |= np.uint32(1 << (s % 32))

    def vertex_words(self, v: int) -> np.ndarray:
        if v >= self.num_vertices or self.words_per_vertex == 0:
            return np.zeros(0, np.uint32)
        w = self.words_per_vertex
        return self.words[v * w:(v + 1) * w]

    def reachable_source_count(self, v: int) -> int:
        words = self.vertex_words(v).astype(np.uint64)
        rem = self.num_sources % 32
        if words.size and rem:
            words = words.copy()
            words[-1] &= (1 << rem) - 1
        return int(sum(bin(int(x)).count("1") for x in words))

    def total_reachable_pairs(self) -> int:
        return int(np.unpackbits(self.words.view(np.uint8)).sum())

    @classmethod
    def from_canonical_distances(cls, num_vertices: int, num_sources: int,
                                 distances: np.ndarray) -> "ReachabilityBitmask":
        """graph.rs:571-646."""
        m = cls.zeroed(num_vertices, num_sources)
        if num_sources == 0 or num_vertices == 0:
            return m
        d = np.asarray(distances, np.uint32).reshape(num_sources, num_vertices)
        bits = (d != UNREACHABLE)
        pad = m.words_per_vertex * 32 - num_sources
        if pad:
            bits = np.vstack([bits, np.zeros((pad, num_vertices), bool)])
        packed = np.packbits(bits.T.reshape(num_vertices, m.words_per_vertex, 32)[..., ::-1],
                             axis=-1)
        m.words = packed.view(">u4").astype(np.uint32).reshape(-1)
        return m

    def __eq__(self, other) -> bool:
        return (isinstance(other, ReachabilityBitmask)
                and self.num_vertices == other.num_vertices
                and self.num_sources == other.num_sources
                and np.array_equal(self.words, other.words))


class GpuBfsMethod(enum.IntEnum):
    """crates/gpu_bfs/src/engine.rs:33-53 (same names and order)."""
    NaiveSequential = 0
    BatchedDenseSpMM = 1
    BitParallel32 = 2
    BitParallel64 = 3
    BitParallel64Pull = 4
    BooleanReachability = 5
    PushPullAdaptive = 6
    SparseQueue = 7
    SparseBitParallel64 = 8
    MultiWordBitParallel = 9
    IndirectMacroBatch = 10
    IndirectSparseQueuePush = 11
    MultiWordBitParallelPush = 12
    WorkgroupPersistentBfs = 13
    Auto = 14


PATH_NAMES = {0: "none", 1: "push", 2: "pull", 3: "hybrid", 4: "cta"}


class DeviceGraph:
    """A graph uploaded to HBM (CSR + CSC) and owned by one engine."""

    def __init__(self, engine: "GpuBfsEngine", graph: CsrGraph):
        self._engine = engine
        self.graph = graph
        h = C.c_void_p()
        rc = _native.lib().msbfs_graph_create(engine._h, graph.num_vertices, graph.num_edges,
                                              _ptr(graph.row_offsets), _ptr(graph.col_indices),
                                              C.byref(h))
        engine._check(rc)
        self._h = h

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        V, E, md, sym = C.c_size_t(), C.c_size_t(), C.c_uint32(), C.c_int()
        _native.lib().msbfs_graph_info(self._h, C.byref(V), C.byref(E), C.byref(md),
                                       C.byref(sym))
        return {"num_vertices": V.value, "num_edges": E.value, "max_degree": md.value,
                "symmetric": bool(sym.value)}

    def close(self) -> None:
        if self._h:
            _native.lib().msbfs_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuBfsEngine:
    """GB300 counterpart of GpuBfsEngine (crates/gpu_bfs/src/engine.rs:57-490).

    Graphs passed to ``run_*`` are uploaded once per engine and kept resident
    (keyed by object identity; CsrGraph arrays are read-only).
    """

    def __init__(self, method: GpuBfsMethod = GpuBfsMethod.Auto, device: int = 0):
        h = C.c_void_p()
        rc = _native.lib().msbfs_engine_create(int(device), int(method), C.byref(h))
        if rc:
            raise BfsError(rc, "engine creation failed (no CUDA device?)")
        self._h = h
        self._method = GpuBfsMethod(method)
        self._graphs: dict = {}
        self._lock = threading.Lock()
        self.last_stats: dict = {}

    # -- lifecycle ------------------------------------------------------------
    def close(self) -> None:
        for dg in list(self._graphs.values()):
            dg.close()
        self._graphs.clear()
        if self._h:
            _native.lib().msbfs_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        if rc:
            msg = _native.lib().msbfs_engine_last_error(self._h)
            raise BfsError(rc, msg.decode() if msg else "")

    # -- reference API --------------------------------------------------------
    def method(self) -> GpuBfsMethod:
        return self._method

    @staticmethod
    def select_auto_method(graph: CsrGraph, num_sources: int) -> GpuBfsMethod:
        """engine.rs:157-198."""
        return GpuBfsMethod(_native.lib().msbfs_select_auto_method(
            graph.num_vertices, graph.num_edges, _ptr(graph.row_offsets), int(num_sources)))

    def resolve_method(self, graph: CsrGraph, sources) -> GpuBfsMethod:
        if self._method == GpuBfsMethod.Auto:
            return self.select_auto_method(graph, len(sources))
        return self._method

    def set_tuning(self, max_words_per_pass: int = 0, alpha: int = 0, beta: int = 0) -> None:
        self._check(_native.lib().msbfs_engine_set_tuning(self._h, max_words_per_pass, alpha,
                                                          beta))

    def autotune(self, graph: CsrGraph, sources, cache_path: Optional[str] = None) -> dict:
        """Tunes the level path's settings for the graph's class and this
        source count (msbfs_engine_autotune) and applies them; returns the
        chosen settings, the tuned and default call times and the class."""
        src = _u32(sources)
        dg = self.upload(graph)
        t = _native.Tuning()
        rc = _native.lib().msbfs_engine_autotune(
            self._h, dg.handle, _ptr(src), src.size,
            cache_path.encode() if cache_path else None, C.byref(t))
        self._check(rc)
        return t.as_dict()

    def set_level_cap(self, max_levels: int) -> None:
        """Stops a level-synchronous pass after ``max_levels`` levels with
        BfsError code 4 (Timeout); 0 restores the default (V + 2)."""
        self._check(_native.lib().msbfs_engine_set_level_cap(self._h, int(max_levels)))

    def set_profiling(self, level: int) -> None:
        """0 off, 1 per-level records with work counters (device timers), 2
        records + host-driven level loop with CUDA events around every launch,
        3 as 2 with the production kernels (durations, no work counters)."""
        self._check(_native.lib().msbfs_engine_set_profiling(self._h, int(level)))

    def level_log(self) -> list:
        n = C.c_size_t()
        _native.lib().msbfs_engine_level_log(self._h, None, 0, C.byref(n))
        recs = (_native.LevelRecord * max(1, n.value))()
        _native.lib().msbfs_engine_level_log(self._h, recs, n.value, C.byref(n))
        return [recs[i].as_dict() for i in range(n.value)]

    def set_stream(self, cuda_stream_handle: int) -> None:
        self._check(_native.lib().msbfs_engine_set_stream(self._h,
                                                          C.c_void_p(cuda_stream_handle)))

    def upload(self, graph: CsrGraph) -> DeviceGraph:
        with self._lock:
            key = id(graph)
            dg = self._graphs.get(key)
            if dg is not None and dg.graph is graph:
                return dg
            dg = DeviceGraph(self, graph)
            self._graphs[key] = dg
            weakref.finalize(graph, self._drop_graph, key)
            return dg

    def _drop_graph(self, key) -> None:
        dg = self._graphs.pop(key, None)
        if dg is not None:
            dg.close()

    def run_ms_bfs(self, graph: CsrGraph, sources) -> np.ndarray:
        """BfsEngine::run_ms_bfs: u32 array of len(sources) * V, dist[s*V + v]."""
        return self.run_ms_bfs_with_method(self._method, graph, sources)

    def run_ms_bfs_into(self, graph: CsrGraph, sources, out: np.ndarray) -> None:
        """GpuBfsEngine::run_ms_bfs_into (engine.rs:219-298) into a caller buffer."""
        self._run(self._method, graph, sources, out)

    def run_ms_bfs_with_method(self, method: GpuBfsMethod, graph: CsrGraph,
                               sources) -> np.ndarray:
        """GpuBfsEngine::run_ms_bfs_with_method (engine.rs:300-405)."""
        src = _u32(sources)
        out = np.empty(src.size * graph.num_vertices, np.uint32)
        self._run(method, graph, src, out)
        return out

    def _run(self, method, graph: CsrGraph, sources, out: np.ndarray) -> None:
        src = _u32(sources)
        if src.size == 0:
            self.last_stats = {}
            return
        if out.dtype != np.uint32 or not out.flags.c_contiguous or \
                out.size != src.size * graph.num_vertices:
            raise ValueError("out must be a contiguous u32 array of len(sources) * V")
        dg = self.upload(graph) if graph.num_vertices else None
        st = Stats()
        if dg is None:
            # V == 0 with S > 0: same error as the reference (engine.rs:233-238).
            raise BfsError(2, f"Source vertex {int(src[0])} at index 0 exceeds graph "
                              f"vertex count 0")
        rc = _native.lib().msbfs_run_ms_bfs_with_method(self._h, int(method), dg.handle,
                                                        _ptr(src), src.size, _ptr(out),
                                                        C.byref(st))
        self._check(rc)
        self.last_stats = st.as_dict()

    def run_ms_bfs_device(self, graph: CsrGraph, sources, out_ptr: int,
                          method: Optional[GpuBfsMethod] = None) -> None:
        """Queues a run writing S*V u32 to device pointer ``out_ptr``; returns
        immediately (call ``synchronize``)."""
        src = _u32(sources)
        dg = self.upload(graph)
        m = self._method if method is None else method
        rc = _native.lib().msbfs_run_ms_bfs_device(self._h, int(m), dg.handle, _ptr(src),
                                                   src.size, C.c_void_p(out_ptr))
        self._check(rc)

    def synchronize(self) -> dict:
        st = Stats()
        self._check(_native.lib().msbfs_engine_synchronize(self._h, C.byref(st)))
        self.last_stats = st.as_dict()
        return self.last_stats

    def run_ms_reachability(self, graph: CsrGraph, sources) -> ReachabilityBitmask:
        """GpuBfsEngine::run_ms_reachability (engine.rs:420-479)."""
        src = _u32(sources)
        m = ReachabilityBitmask.zeroed(graph.num_vertices, src.size)
        if src.size == 0 or graph.num_vertices == 0:
            return m
        dg = self.upload(graph)
        st = Stats()
        rc = _native.lib().msbfs_run_reachability(self._h, dg.handle, _ptr(src), src.size,
                                                  _ptr(m.words), C.byref(st))
        self._check(rc)
        self.last_stats = st.as_dict()
        return m

    def run_reachability(self, graph: CsrGraph, sources) -> ReachabilityBitmask:
        """ReachabilityEngine::run_reachability (crates/core/src/lib.rs:65-88)."""
        return self.run_ms_reachability(graph, sources)

    def traversed_edges_device(self, graph: CsrGraph, dist_ptr: int, num_sources: int) -> int:
        dg = self.upload(graph)
        out = C.c_uint64()
        self._check(_native.lib().msbfs_traversed_edges_device(
            self._h, dg.handle, C.c_void_p(dist_ptr), num_sources, C.byref(out)))
        return out.value

    def run_ms_bfs_stats(self, graph: CsrGraph, sources) -> np.ndarray:
        """Per-source eccentricity / reached count / distance sum, computed on
        the device without forming the S*V matrix (msbfs_run_ms_bfs_stats)."""
        src = _u32(sources)
        out = np.zeros(src.size, SOURCE_STATS_DTYPE)
        if src.size == 0:
            return out
        dg = self.upload(graph)
        st = Stats()
        rc = _native.lib().msbfs_run_ms_bfs_stats(self._h, dg.handle, _ptr(src), src.size,
                                                  out.ctypes.data_as(C.c_void_p), C.byref(st))
        self._check(rc)
        self.last_stats = st.as_dict()
        return out

    def set_sm_share(self, percent: int) -> None:
        """Caps the persistent kernels' grids at ``percent`` of the resident
        capacity (msbfs_engine_set_sm_share)."""
        self._check(_native.lib().msbfs_engine_set_sm_share(self._h, int(percent)))


SOURCE_STATS_DTYPE = np.dtype(_native.SOURCE_STATS_DTYPE)


class ServerTicket:
    __slots__ = ("id", "out", "mode", "sources")

    def __init__(self, tid, out, mode, sources):
        self.id, self.out, self.mode, self.sources = tid, out, mode, sources


class BfsServer:
    """Served form (msbfs_server_*): a resident graph, a request queue and a
    scheduler that packs requests into shared traversals on ``slots``
    concurrent engines. ``submit`` returns at once; ``wait`` returns the
    result (rows: u32 array of S*V; stats: SOURCE_STATS_DTYPE array) and the
    request's latency record."""

    ROWS, STATS = 0, 1

    def __init__(self, graph: "CsrGraph", slots: int = 2, max_sources_per_launch: int = 512,
                 hbm_budget_bytes: int = 0, method: GpuBfsMethod = GpuBfsMethod.Auto,
                 device: int = 0, express_slots: int = 0, small_sources: int = 64,
                 general_sm_percent: int = 100):
        cfg = _native.ServerConfig(slots, max_sources_per_launch, hbm_budget_bytes, int(method),
                                   express_slots, small_sources, general_sm_percent, 0)
        h = C.c_void_p()
        self.graph = graph
        self.V = graph.num_vertices
        _check(_native.lib().msbfs_server_create(device, graph.num_vertices, graph.num_edges,
                                                 _ptr(graph.row_offsets),
                                                 _ptr(graph.col_indices), C.byref(cfg),
                                                 C.byref(h)), "msbfs_server_create failed")
        self._h = h

    def submit(self, sources, mode: int = STATS, out: Optional[np.ndarray] = None) -> ServerTicket:
        src = _u32(sources)
        if out is None:
            out = (np.empty(src.size * self.V, np.uint32) if mode == self.ROWS
                   else np.zeros(src.size, SOURCE_STATS_DTYPE))
        t = C.c_uint64()
        rc = _native.lib().msbfs_server_submit(self._h, _ptr(src), src.size, int(mode),
                                               out.ctypes.data_as(C.c_void_p), C.byref(t))
        _check(rc, "submit failed")
        return ServerTicket(t.value, out, mode, src)

    def wait(self, ticket: ServerTicket, timeout_ms: float = -1.0):
        info = _native.RequestInfo()
        rc = _native.lib().msbfs_server_wait(self._h, ticket.id, float(timeout_ms),
                                             C.byref(info))
        _check(rc, "request failed")
        return ticket.out, info.as_dict()

    def counters(self) -> dict:
        """Traversals and kernel launches issued since creation."""
        t, k = C.c_uint64(), C.c_uint64()
        _check(_native.lib().msbfs_server_counters(self._h, C.byref(t), C.byref(k)),
               "counters failed")
        return {"traversals": t.value, "kernel_launches": k.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().msbfs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchedBfs:
    """Many graphs of uneven size, each with its own sources, traversed in one
    persistent launch (msbfs_batch_*). ``items`` is a sequence of
    ``(CsrGraph, sources)``. Results stay on the device until ``result(i)``."""

    ALG_NAMES = {0: "bit_parallel_block", 1: "source_per_bfs", 2: "bit_parallel_vertex_tiles"}

    def __init__(self, items, device: int = 0):
        self._keep = []
        arr = (_native.BatchGraph * max(1, len(items)))()
        for i, (g, src) in enumerate(items):
            s = _u32(src)
            self._keep.append((g, s))
            arr[i].num_vertices = g.num_vertices
            arr[i].num_edges = g.num_edges
            arr[i].row_offsets = _ptr(g.row_offsets)
            arr[i].col_indices = _ptr(g.col_indices)
            arr[i].sources = _ptr(s)
            arr[i].num_sources = s.size
        self._arr = arr
        self._n = len(items)
        h = C.c_void_p()
        _check(_native.lib().msbfs_batch_create(device, C.cast(arr, C.c_void_p), self._n,
                                                C.byref(h)), "msbfs_batch_create failed")
        self._h = h

    def __len__(self):
        return self._n

    def autotune(self, samples_per_class: int = 3, cache_path: Optional[str] = None) -> None:
        _check(_native.lib().msbfs_batch_autotune(
            self._h, samples_per_class, cache_path.encode() if cache_path else None),
            "autotune failed")

    def run(self) -> float:
        """One persistent launch over every graph; returns device ms."""
        ms = C.c_double()
        _check(_native.lib().msbfs_batch_run(self._h, C.byref(ms)), "batch run failed")
        return ms.value

    def run_per_graph(self) -> float:
        """The plain path: one engine call per graph; returns device ms."""
        ms = C.c_double()
        _check(_native.lib().msbfs_batch_run_per_graph(self._h, C.cast(self._arr, C.c_void_p),
                                                       C.byref(ms)), "per-graph run failed")
        return ms.value

    def result(self, i: int) -> np.ndarray:
        g, s = self._keep[i]
        out = np.empty(s.size * g.num_vertices, np.uint32)
        if out.size:
            _check(_native.lib().msbfs_batch_result(self._h, i, _ptr(out)), "result failed")
        return out

    def config(self, i: int) -> dict:
        a, w, prm = C.c_uint32(), C.c_uint32(), C.c_uint32()
        name = C.create_string_buffer(64)
        _check(_native.lib().msbfs_batch_config(self._h, i, C.byref(a), C.byref(w),
                                                C.byref(prm), name, 64))
        return {"class": name.value.decode(), "alg": self.ALG_NAMES.get(a.value, a.value),
                "words": w.value, "param": prm.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().msbfs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ generators
GRAPH500_A, GRAPH500_B, GRAPH500_C, GRAPH500_D = 0.57, 0.19, 0.19, 0.05


def _gen(fn_name: str, *args) -> CsrGraph:
    c = Csr()
    _check(getattr(_native.lib(), fn_name)(*args, C.byref(c)), fn_name)
    V, _, off, idx = _take_csr(c)
    return CsrGraph(V, off, idx)


class Grid2D:
    """Grid2D (generators.rs:18-128) with its Manhattan-distance oracle."""

    def __init__(self, width: int, height: int):
        if width == 0 or height == 0:
            raise ValueError("invalid grid dimensions")
        self.width, self.height = width, height
        self.graph = _gen("msbfs_gen_grid2d", width, height)

    def vertex_id(self, x: int, y: int) -> int:
        return y * self.width + x

    def coordinates(self, v: int):
        return v % self.width, v // self.width

    def manhattan_distance(self, a: int, b: int) -> int:
        (x1, y1), (x2, y2) = self.coordinates(a), self.coordinates(b)
        return abs(x1 - x2) + abs(y1 - y2)

    def ms_bfs_oracle(self, sources) -> np.ndarray:
        v = np.arange(self.width * self.height)
        x, y = v % self.width, v // self.width
        s = np.asarray(sources, np.int64)
        sx, sy = s % self.width, s // self.width
        return (np.abs(x[None, :] - sx[:, None]) + np.abs(y[None, :] - sy[:, None])) \
            .astype(np.uint32).reshape(-1)

    def single_source_oracle(self, source: int) -> np.ndarray:
        return self.ms_bfs_oracle([source])


def generate_grid2d(width: int, height: int) -> CsrGraph:
    return Grid2D(width, height).graph


def generate_erdos_renyi_np(n: int, p: float, seed: int) -> CsrGraph:
    return _gen("msbfs_gen_erdos_renyi_np", n, float(p), seed & (2**64 - 1))


def generate_random_tree(n: int, seed: int) -> CsrGraph:
    return _gen("msbfs_gen_random_tree", n, seed & (2**64 - 1))


def generate_rmat(scale: int, edge_factor: int, a: float, b: float, c: float, d: float,
                  seed: int, directed: bool = False) -> CsrGraph:
    return _gen("msbfs_gen_rmat", scale, edge_factor, a, b, c, d, seed & (2**64 - 1),
                int(directed))


def generate_graph500_rmat(scale: int, edge_factor: int, seed: int) -> CsrGraph:
    return generate_rmat(scale, edge_factor, GRAPH500_A, GRAPH500_B, GRAPH500_C, GRAPH500_D,
                         seed, False)


def empty_graph() -> CsrGraph:
    return CsrGraph(0, [0], [])


def isolated_vertices(n: int) -> CsrGraph:
    return CsrGraph(n, np.zeros(n + 1, np.uint32), [])


def single_vertex() -> CsrGraph:
    return isolated_vertices(1)


def path_graph(n: int) -> CsrGraph:
    return _gen("msbfs_gen_path", n)


def star_graph(n: int) -> CsrGraph:
    return _gen("msbfs_gen_star", n)


def cycle_graph(n: int) -> CsrGraph:
    return _gen("msbfs_gen_cycle", n)


def clique_graph(n: int) -> CsrGraph:
    return _gen("msbfs_gen_clique", n)


def disconnected_cliques(sizes: Sequence[int]) -> CsrGraph:
    arr = (C.c_size_t * max(1, len(sizes)))(*sizes)
    return _gen("msbfs_gen_disconnected_cliques", arr, len(sizes))


def wilson_grid(width: int, height: int, extra_edges: int, seed: int) -> CsrGraph:
    """Uniform spanning tree of a width x height grid (Wilson's algorithm)
    plus ``extra_edges`` distinct non-tree grid edges, symmetrised."""
    return _gen("msbfs_gen_wilson_grid", width, height, extra_edges, seed & (2**64 - 1))


def sample_sources(graph: CsrGraph, count: int, seed: int, min_degree: int = 0) -> np.ndarray:
    """graph_loader.rs:132-190 random strategy: distinct, sorted ascending."""
    out = np.empty(count, np.uint32)
    rc = _native.lib().msbfs_sample_sources(C.byref(graph._as_csr()), count,
                                            seed & (2**64 - 1), min_degree, _ptr(out))
    _check(rc, "not enough eligible vertices")
    return out


class MtxError(BfsError):
    """MtxError of the reference (crates/core/src/error.rs:43-81): ``kind`` is
    the variant name, the other attributes its fields (0 when unused)."""

    KINDS = {1: "Io", 2: "InvalidHeader", 3: "UnsupportedFormat", 4: "InvalidDimensions",
             5: "InvalidCoordinateLine", 6: "ZeroIndex", 7: "IndexOutOfBounds"}

    def __init__(self, err: "_native.MtxErrorInfo"):
        super().__init__(10, err.message.decode(errors="replace"))
        self.kind = self.KINDS.get(err.kind, f"kind {err.kind}")
        self.line_number = err.line_number
        self.row, self.col = err.row, err.col
        self.max_rows, self.max_cols = err.max_rows, err.max_cols


def _mtx_result(rc: int, c: Csr, err) -> CsrGraph:
    if rc == 10:
        raise MtxError(err)
    _check(rc, "Matrix Market read failed")
    V, _, off, idx = _take_csr(c)
    return CsrGraph(V, off, idx)


def parse_mtx(text) -> CsrGraph:
    """MtxReader::parse (crates/core/src/mtx.rs:124) of Matrix Market text."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    c, err = Csr(), _native.MtxErrorInfo()
    rc = _native.lib().msbfs_mtx_parse(data, len(data), C.byref(c), C.byref(err))
    return _mtx_result(rc, c, err)


def read_mtx(path) -> CsrGraph:
    """Reads a Matrix Market (.mtx) file into a CsrGraph."""
    c, err = Csr(), _native.MtxErrorInfo()
    rc = _native.lib().msbfs_mtx_read(str(path).encode(), C.byref(c), C.byref(err))
    return _mtx_result(rc, c, err)
