"""The allocation-free entry point, through the C ABI (GPU).

msbfs_run_cta_noalloc serves callers that must not call cudaMalloc: hosts
whose device memory all belongs to their own pool allocator, and services
that reserve every byte at start so that no request can fail later for want
of memory. It keeps its scratch in a fixed device array inside the library
and takes device-resident inputs and outputs. Here the test allocates those
buffers itself (with torch) and checks the distances bit for bit (integer
output: no tolerance) against the CPU oracle and against msbfs_run_ms_bfs,
on two calls in a row that share the fixed array: graphs well inside the
limit, a call of more than 65,536 sources (two chunks through the array),
and a graph of exactly MSBFS_NOALLOC_MAX_VERTICES vertices. The file name
sorts last so that a run stopping at the first failure has run every other
test before this one.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_same

pytestmark = pytest.mark.gpu

MSBFS_ERR_SOURCE_OOB = 1
MSBFS_ERR_SCRATCH_TOO_SMALL = 9
MAX_VERTICES = 1048576  # MSBFS_NOALLOC_MAX_VERTICES
CHUNK = 65536  # sources per chunk through the fixed array


def _call(lib, native, n_vertices, ro_ptr, ci_ptr, src, out_ptr):
    return lib.msbfs_run_cta_noalloc(0, n_vertices, C.c_void_p(ro_ptr), C.c_void_p(ci_ptr),
                                     src.ctypes.data_as(native._native.u32p), src.size,
                                     C.c_void_p(out_ptr), None)


def _run_noalloc(torch, lib, native, g, src):
    ro = torch.from_numpy(g.row_offsets.view(np.int32).copy()).cuda()
    ci = torch.from_numpy(g.col_indices.view(np.int32).copy()).cuda()
    out = torch.full((src.size * g.num_vertices,), 7, dtype=torch.int32, device="cuda")
    rc = _call(lib, native, g.num_vertices, ro.data_ptr(), ci.data_ptr(), src, out.data_ptr())
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32)


def _check(torch, lib, native, oracle, eng, g, src, label):
    got = _run_noalloc(torch, lib, native, g, src)
    want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, src)
    assert_same(got, want, g, src, f"{label} vs oracle")
    assert_same(got, eng.run_ms_bfs(g, src), g, src, f"{label} vs msbfs_run_ms_bfs")


def test_noalloc_matches_oracle_and_engine_on_two_calls_in_a_row(native, oracle):
    torch = pytest.importorskip("torch")
    lib = native._native.lib()
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        graphs = [(native.wilson_grid(60, 50, 80, 5), (11, 12)),
                  (native.generate_graph500_rmat(12, 8, 3), (13, 14))]
        for g, seeds in graphs:
            for seed in seeds:  # two calls in a row on the shared scratch
                src = np.random.default_rng(seed).integers(0, g.num_vertices, 300)
                _check(torch, lib, native, oracle, eng, g, src.astype(np.uint32),
                       f"V={g.num_vertices} seed={seed}")
    finally:
        eng.close()


def test_noalloc_more_sources_than_one_chunk(native, oracle):
    """70,000 sources: the entry point copies them through its fixed array in
    two chunks, one after the other on the stream."""
    torch = pytest.importorskip("torch")
    lib = native._native.lib()
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        g = native.wilson_grid(20, 16, 12, 8)
        src = np.random.default_rng(70).integers(0, g.num_vertices, CHUNK + 4464)
        for k in range(2):  # two calls in a row
            _check(torch, lib, native, oracle, eng, g, np.roll(src, k).astype(np.uint32),
                   f"{src.size} sources, call {k}")
    finally:
        eng.close()


def test_noalloc_at_the_vertex_limit(native, oracle):
    """A 1024 x 1024 grid has exactly MSBFS_NOALLOC_MAX_VERTICES vertices:
    its visited bitmap and queue halves fit one block and a queue slab fits
    the fixed array."""
    torch = pytest.importorskip("torch")
    lib = native._native.lib()
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        g = native.generate_grid2d(1024, 1024)
        assert g.num_vertices == MAX_VERTICES
        for src in (np.array([0, MAX_VERTICES - 1, 512 * 1024 + 512], np.uint32),
                    np.array([1023, 1024 * 1023, 77, 300000, 5], np.uint32)):
            _check(torch, lib, native, oracle, eng, g, src, f"grid 1024^2 {src.tolist()}")
    finally:
        eng.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(native):
    lib = native._native.lib()
    src = np.zeros(1, np.uint32)
    # Rejected before any pointer is used or any work is queued.
    rc = _call(lib, native, MAX_VERTICES + 1, 16, 16, src, 16)
    assert rc == MSBFS_ERR_SCRATCH_TOO_SMALL
    rc = _call(lib, native, 10, 16, 16, np.array([10], np.uint32), 16)
    assert rc == MSBFS_ERR_SOURCE_OOB
