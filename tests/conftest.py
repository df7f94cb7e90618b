"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden" / "known_answers.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def native():
    import __graft_entry__  # noqa: F401  (build helpers)
    from webgpu_bfs_gb300 import build as b
    b.build_native()
    import webgpu_bfs_gb300 as m
    return m


@pytest.fixture(scope="session")
def gpu_engine(native):
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    yield eng
    eng.close()


def case_graph(native, case):
    return native.CsrGraph(case["num_vertices"], case["row_offsets"], case["col_indices"])


def assert_same(got, want, graph=None, sources=None, label=""):
    """Bit-exact comparison with a first-mismatch diagnostic like the
    reference's tests/common/diagnostics.rs."""
    got = np.asarray(got, np.uint32)
    want = np.asarray(want, np.uint32)
    assert got.shape == want.shape, f"{label}: shape {got.shape} != {want.shape}"
    if np.array_equal(got, want):
        return
    bad = np.flatnonzero(got != want)
    i = int(bad[0])
    msg = f"{label}: {bad.size} mismatches ({100.0 * bad.size / got.size:.3f}%)"
    if graph is not None and sources is not None and graph.num_vertices:
        V = graph.num_vertices
        s, v = divmod(i, V)
        nb = graph.col_indices[graph.row_offsets[v]:graph.row_offsets[v + 1]][:16]
        msg += (f"; first at s_idx={s} (source {int(sources[s])}) v={v}: "
                f"expected {int(want[i])}, got {int(got[i])}, degree {nb.size}, "
                f"neighbours {nb.tolist()}")
    raise AssertionError(msg)
