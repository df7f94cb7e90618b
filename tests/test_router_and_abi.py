"""Auto router parity with the reference and C-ABI export checks (no GPU)."""
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def _hub(native, max_deg):
    """make_graph_with_max_degree (crates/gpu_bfs/src/engine.rs:496-500)."""
    nv = max_deg + 2
    return native.CsrGraph.from_edge_list(nv, [(0, v) for v in range(1, max_deg + 1)])


def test_select_auto_empty_and_zero_sources(native):
    M = native.GpuBfsMethod
    assert native.GpuBfsEngine.select_auto_method(native.empty_graph(), 64) == M.NaiveSequential
    assert native.GpuBfsEngine.select_auto_method(_hub(native, 5), 0) == M.NaiveSequential


def test_select_auto_low_degree(native):
    """engine.rs:514-535."""
    M = native.GpuBfsMethod
    for deg in (0, 1, 4, 7, 8):
        g = _hub(native, deg)
        assert g.max_degree() == deg
        for s in (1, 2, 16, 31, 32, 63, 64, 256, 512, 1024, 2048):
            assert native.GpuBfsEngine.select_auto_method(g, s) == M.WorkgroupPersistentBfs
    g9 = _hub(native, 9)
    assert native.GpuBfsEngine.select_auto_method(g9, 1) == M.SparseQueue
    assert native.GpuBfsEngine.select_auto_method(g9, 16) == M.BitParallel32
    assert native.GpuBfsEngine.select_auto_method(g9, 32) == M.BitParallel64
    assert native.GpuBfsEngine.select_auto_method(g9, 64) == M.MultiWordBitParallel


def test_select_auto_intermediate(native):
    """engine.rs:538-583."""
    M = native.GpuBfsMethod
    for deg in (9, 16, 32, 33, 50, 64, 100, 127):
        g = _hub(native, deg)
        sel = native.GpuBfsEngine.select_auto_method
        assert sel(g, 1) == M.SparseQueue
        assert sel(g, 16) == M.BitParallel32
        assert sel(g, 32) == M.BitParallel64 and sel(g, 63) == M.BitParallel64
        for s in (64, 512, 2048):
            assert sel(g, s) == M.MultiWordBitParallel


def test_select_auto_hubs(native):
    """engine.rs:586-605."""
    M = native.GpuBfsMethod
    for deg in (128, 256, 1024, 38625):
        g = _hub(native, deg)
        for s in (1, 2, 16, 32, 63, 64, 128, 256, 384, 512, 1024, 2048):
            assert native.GpuBfsEngine.select_auto_method(g, s) == M.IndirectSparseQueuePush


def test_library_exports_every_declared_symbol(native):
    header = (ROOT / "include" / "msbfs.h").read_text()
    declared = set(re.findall(r"\b(msbfs_[a-z0-9_]+)\s*\(", header))
    declared -= {"msbfs_method"}
    lib = native._native.lib()
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, f"missing exports: {missing}"
    assert declared == set(native._native.SIGNATURES), "ctypes table out of sync with header"


def test_engine_creation_without_gpu_fails_cleanly(native):
    """On a machine without a CUDA device the engine reports NoDevice instead
    of falling back to the CPU."""
    import ctypes as C
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    h = C.c_void_p()
    rc = native._native.lib().msbfs_engine_create(0, 14, C.byref(h))
    assert rc == 8  # MSBFS_ERR_NO_DEVICE


def test_csr_one_shot_entry_validates_before_device(native):
    """Empty source list succeeds without touching a device (engine.rs:228-231)."""
    src = np.zeros(0, np.uint32)
    assert src.size == 0
