"""The allocation-free entry point against the engine, through the C ABI (GPU).

msbfs_run_cta_noalloc serves callers that cannot call cudaMalloc -- code that
runs under an active stream capture, or hosts whose device memory belongs to
their own pool allocator. It keeps its scratch in a fixed device array inside
the library and takes device-resident inputs and outputs. Here the test
allocates those buffers itself (with torch) and checks, on two calls in a
row, that the distances are bit-identical to msbfs_run_ms_bfs (integer
output: no tolerance). The file name sorts last so that a run stopping at
the first failure has run every other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MSBFS_ERR_SOURCE_OOB = 1
MSBFS_ERR_SCRATCH_TOO_SMALL = 9
MAX_VERTICES = 1048576  # MSBFS_NOALLOC_MAX_VERTICES


def _call(lib, native, n_vertices, ro_ptr, ci_ptr, src, out_ptr):
    return lib.msbfs_run_cta_noalloc(0, n_vertices, C.c_void_p(ro_ptr), C.c_void_p(ci_ptr),
                                     src.ctypes.data_as(native._native.u32p), src.size,
                                     C.c_void_p(out_ptr), None)


def test_noalloc_matches_engine_on_two_calls_in_a_row(native):
    torch = pytest.importorskip("torch")
    lib = native._native.lib()
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        graphs = [(native.wilson_grid(60, 50, 80, 5), (11, 12)),
                  (native.generate_graph500_rmat(12, 8, 3), (13, 14))]
        for g, seeds in graphs:
            ro = torch.from_numpy(g.row_offsets.view(np.int32).copy()).cuda()
            ci = torch.from_numpy(g.col_indices.view(np.int32).copy()).cuda()
            for seed in seeds:  # two calls in a row on the shared scratch
                src = np.random.default_rng(seed).integers(0, g.num_vertices, 300)
                src = src.astype(np.uint32)
                out = torch.full((src.size * g.num_vertices,), 7, dtype=torch.int32,
                                 device="cuda")
                rc = _call(lib, native, g.num_vertices, ro.data_ptr(), ci.data_ptr(), src,
                           out.data_ptr())
                assert rc == 0
                torch.cuda.synchronize()
                got = out.cpu().numpy().view(np.uint32)
                want = eng.run_ms_bfs(g, src)
                assert np.array_equal(got, want), f"V={g.num_vertices} seed={seed}"
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
