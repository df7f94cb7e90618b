"""Bit-exact parity at the benchmarked configurations' full sizes (GPU).

The graphs, sources and seeds are bench.py's own workloads, so these are the
inputs the reported numbers are measured on: R-MAT scale 22 at S=64 and
S=512 (the headline), the 339 x 338 Wilson road graph with 5,000 extra edges
at S=1, 256 and 2,048, the 64 x 64 grid at S=64, the served configuration's
two resident graphs (R-MAT scale 24 and the 1448 x 1448 road graph), and a
100-graph slice of the 1,000-graph batched configuration. Rows are compared
byte for byte with the CPU oracle (threaded FIFO, the reference's Rayon path
restated): every row where the oracle finishes in seconds, an evenly spread
sample of rows on the R-MAT graphs. Integer output: no tolerance.

Reference counterparts: crates/cli/src/verify.rs:28-60 (every engine's
output checked against the CPU engine on the benchmarked graph) and
crates/gpu_bfs/tests/m10_e2e_parity.rs:502-600 (parity on the real dataset).
"""
import numpy as np
import pytest

import bench
from conftest import assert_same

pytestmark = pytest.mark.gpu


def _spread(S, n):
    """n source indices spread evenly over 0..S-1, first and last included."""
    return sorted(set(np.linspace(0, S - 1, min(n, S)).round().astype(int).tolist()))


def _check_rows(oracle, g, src, rows_of, idx, label):
    """rows_of(i) -> row i of the GPU output; compares rows `idx`."""
    V = g.num_vertices
    want = oracle.ms_bfs_threaded(V, g.row_offsets, g.col_indices, src[idx])
    for k, i in enumerate(idx):
        assert_same(rows_of(i), want[k * V:(k + 1) * V], g, src[i:i + 1],
                    f"{label} row {i} (source {int(src[i])})")


@pytest.fixture(scope="module")
def rmat22(native):
    return bench.make_graph(native, bench.WORKLOADS["rmat22_s512"])


@pytest.mark.parametrize("workload", ["rmat22_s64", "rmat22_s512"])
def test_rmat22_rows_match_oracle(native, oracle, rmat22, workload):
    torch = pytest.importorskip("torch")
    spec = bench.WORKLOADS[workload]
    g, S = rmat22, spec["S"]
    V = g.num_vertices
    src = native.sample_sources(g, S, spec["seed"], min_degree=1)  # the bench's sources
    idx = _spread(S, 64 if S <= 64 else 40)
    out = torch.empty(S * V, dtype=torch.int32, device="cuda")
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        for method in ("Auto", "MultiWordBitParallel", "BitParallel64"):
            out.fill_(7)
            eng.run_ms_bfs_device(g, src, out.data_ptr(), native.GpuBfsMethod[method])
            st = eng.synchronize()
            if method == "Auto":
                # the headline path: device-switched push/pull
                assert st["path"] == 3 and st["push_levels"] >= 1 and st["pull_levels"] >= 1
            _check_rows(oracle, g, src, lambda i: out[i * V:(i + 1) * V].cpu().numpy(), idx,
                        f"{workload}/{method}")
    finally:
        eng.close()


@pytest.mark.parametrize("workload", ["road_s1", "road_s256", "road_s2048"])
def test_road_339x338_all_rows_match_oracle(native, oracle, workload):
    spec = bench.WORKLOADS[workload]
    g = bench.make_graph(native, spec)
    assert g.num_vertices == 339 * 338
    src = native.sample_sources(g, spec["S"], spec["seed"], min_degree=1)
    want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, src)
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        got = eng.run_ms_bfs(g, src)
        assert eng.last_stats["path"] == 4  # the router's road choice: CTA per source
        assert_same(got, want, g, src, f"{workload}/Auto")
        if spec["S"] >= 256:
            # the level path on a ~1,000-level graph: distances past the 8
            # level planes are written directly
            got = eng.run_ms_bfs_with_method(native.GpuBfsMethod.PushPullAdaptive, g, src)
            assert eng.last_stats["levels"] > 256
            assert_same(got, want, g, src, f"{workload}/PushPullAdaptive")
    finally:
        eng.close()


def test_grid64_s64_matches_manhattan_and_oracle(native, oracle):
    spec = bench.WORKLOADS["grid64_s64"]
    g = bench.make_graph(native, spec)
    src = native.sample_sources(g, spec["S"], spec["seed"], min_degree=1)
    grid = native.Grid2D(64, 64)
    manhattan = grid.ms_bfs_oracle(src)
    want = oracle.ms_bfs_bit_parallel(g.num_vertices, g.row_offsets, g.col_indices, src)
    assert np.array_equal(manhattan, want)
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        for method in ("Auto", "BitParallel64", "MultiWordBitParallel"):
            got = eng.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
            assert_same(got, want, g, src, f"grid64/{method}")
    finally:
        eng.close()


def test_served_graphs_rows_match_oracle(native, oracle):
    """The served configuration's resident graphs: R-MAT scale 24 (level
    path, sampled rows) and the 1448 x 1448 road graph (CTA path with a
    thread-block cluster per source, all rows)."""
    torch = pytest.importorskip("torch")
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        g = bench.make_graph(native, bench.WORKLOADS["served_rmat24"]["graph"])
        V = g.num_vertices
        assert V == 1 << 24
        src = native.sample_sources(g, 64, 24, min_degree=1)
        out = torch.empty(src.size * V, dtype=torch.int32, device="cuda")
        eng.run_ms_bfs_device(g, src, out.data_ptr())
        assert eng.synchronize()["path"] == 3
        _check_rows(oracle, g, src, lambda i: out[i * V:(i + 1) * V].cpu().numpy(),
                    _spread(64, 16), "rmat24 S=64")
        del out, g
        g = bench.make_graph(native, bench.WORKLOADS["served_road1448"]["graph"])
        src = native.sample_sources(g, 8, 1448, min_degree=1)
        got = eng.run_ms_bfs(g, src)
        assert eng.last_stats["path"] == 4 and eng.last_stats["cta_cluster"] >= 2
        want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, src)
        assert_same(got, want, g, src, "road1448 S=8")
    finally:
        eng.close()


def test_batched1000_slice_matches_oracle(native, oracle):
    """Every 10th graph of the batched configuration (60 Erdos-Renyi, 30
    road-like grids, 10 R-MAT scale 16), autotuned, one persistent launch."""
    items = bench.make_batch(native, bench.WORKLOADS["batched1000"])[::10]
    assert len(items) == 100
    b = native.BatchedBfs(items)
    try:
        b.autotune(samples_per_class=2)
        b.run()
        for i, (g, s) in enumerate(items):
            want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, s)
            assert_same(b.result(i), want, g, s, f"batched graph {i} {b.config(i)}")
    finally:
        b.close()
