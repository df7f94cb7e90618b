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


class MtxOracleError(ValueError):
    """A rejected Matrix Market text: ``kind`` names the MtxError variant
    (crates/core/src/error.rs:43-81), ``line`` its line number (0: none)."""

    def __init__(self, kind: str, line: int, message: str):
        super().__init__(message)
        self.kind, self.line = kind, line


def _rust_usize(tok: str):
    """usize::from_str: optional '+', ASCII digits, 64-bit range."""
    body = tok[1:] if tok.startswith("+") else tok
    if tok == "":
        return None, "cannot parse integer from empty string"
    if body == "" or not all("0" <= ch <= "9" for ch in body):
        return None, "invalid digit found in string"
    v = int(body)
    if v >= 1 << 64:
        return None, "number too large to fit in target type"
    return v, None


def mtx_parse(text: str):
    """MtxReader::parse (crates/core/src/mtx.rs:124-275), line by line like the
    reference -> (V, row_offsets, col_indices); raises MtxOracleError."""
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()  # BufRead::lines yields no empty line after the last newline
    i = 0

    def nxt():
        nonlocal i
        if i >= len(lines):
            i += 1
            return None
        s = lines[i].strip(" \t\r\n\v\f")
        i += 1
        return s

    while True:
        s = nxt()
        if s is None:
            raise MtxOracleError("InvalidHeader", i, f"Invalid Matrix Market header at line {i}: "
                                 "Empty input: no MatrixMarket header found")
        if s:
            break
    t = s.split()
    hdr = f"Invalid Matrix Market header at line {i}: "
    if len(t) != 5:
        raise MtxOracleError("InvalidHeader", i, hdr + f"Expected 5 tokens in header line, "
                             f"found {len(t)}: '{s}'")
    if t[0].lower() != "%%matrixmarket":
        raise MtxOracleError("InvalidHeader", i, hdr + f"Missing '%%MatrixMarket' banner: "
                             f"'{t[0]}'")
    if t[1].lower() != "matrix":
        raise MtxOracleError("InvalidHeader", i, hdr + f"Unsupported object '{t[1]}', only "
                             "'matrix' is supported")
    fmt, field, sym = t[2].lower(), t[3].lower(), t[4].lower()
    if fmt == "array":
        raise MtxOracleError("UnsupportedFormat", 0, "Unsupported Matrix Market format "
                             "'array': only sparse 'coordinate' format is supported")
    if fmt != "coordinate":
        raise MtxOracleError("InvalidHeader", i, hdr + f"Unknown format '{fmt}'")
    if field not in ("pattern", "real", "integer", "complex"):
        raise MtxOracleError("InvalidHeader", i, hdr + f"Unknown field '{field}'")
    if sym not in ("general", "symmetric", "skew-symmetric", "hermitian"):
        raise MtxOracleError("InvalidHeader", i, hdr + f"Unknown symmetry '{sym}'")
    symmetric = sym != "general"
    while True:
        s = nxt()
        if s is None:
            raise MtxOracleError("InvalidDimensions", i, f"Invalid dimensions at line {i}: "
                                 "Unexpected end of file while searching for dimension line")
        if s and not s.startswith("%"):
            break
    t = s.split()
    dim = f"Invalid dimensions at line {i}: "
    if len(t) != 3:
        raise MtxOracleError("InvalidDimensions", i, dim + "Expected 3 integer tokens (rows "
                             f"cols nnz), got {len(t)}: '{s}'")
    vals = []
    for name, tok in zip(("rows", "cols", "nnz"), t):
        v, why = _rust_usize(tok)
        if why:
            raise MtxOracleError("InvalidDimensions", i, dim + f"Failed to parse {name} count "
                                 f"'{tok}': {why}")
        vals.append(v)
    rows, cols, _ = vals
    if symmetric and rows != cols:
        raise MtxOracleError("InvalidDimensions", i, dim + "Symmetric matrix must be square, "
                             f"but got {rows} rows and {cols} cols")
    edges = []
    while i < len(lines):
        s = nxt()
        if not s or s.startswith("%"):
            continue
        t = s.split()
        if len(t) < 2:
            raise MtxOracleError("InvalidCoordinateLine", i,
                                 f"Invalid coordinate entry at line {i}: '{s}'")
        r, e1 = _rust_usize(t[0])
        c, e2 = _rust_usize(t[1])
        if e1 or e2:
            raise MtxOracleError("InvalidCoordinateLine", i,
                                 f"Invalid coordinate entry at line {i}: '{s}'")
        if r == 0 or c == 0:
            raise MtxOracleError("ZeroIndex", i, "Matrix Market coordinates are 1-based, but "
                                 f"found 0 at line {i}: row={r}, col={c}")
        if r > rows or c > cols:
            raise MtxOracleError("IndexOutOfBounds", i, f"Coordinate out of bounds at line {i}: "
                                 f"entry ({r}, {c}) exceeds matrix dimensions ({rows}, {cols})")
        if r == c:
            continue
        edges.append((r - 1, c - 1))
        if symmetric:
            edges.append((c - 1, r - 1))
    V = max(rows, cols)
    ro, ci = csr_from_edge_list(V, edges if edges else np.zeros((0, 2), np.uint32))
    return V, ro, ci
