"""CPU checks of bench.py's host-side pieces: the served request stream, the
Poisson arrivals, the latency summary and the algorithmic-bytes model of a
level (the roofline's numerator)."""
import numpy as np

import bench


def test_request_stream_shapes(native):
    g = native.wilson_grid(80, 60, 90, 5)
    reqs = bench.make_requests(g, 200, 11)
    sizes = {int(r.size) for r in reqs}
    assert sizes <= set(bench.SERVED_SIZES) and len(sizes) >= 4
    deg = np.diff(g.row_offsets.astype(np.int64))
    for r in reqs:
        assert np.all(np.diff(r.astype(np.int64)) > 0)  # distinct, sorted
        assert np.all(deg[r] >= 1)
    again = bench.make_requests(g, 200, 11)
    assert all(np.array_equal(a, b) for a, b in zip(reqs, again))  # seeded


def test_small_request_workload_spec(native):
    spec = bench.WORKLOADS["served_rmat22_small"]
    assert max(spec["sizes"]) <= 64 and spec["server"]["express_slots"] == 0
    # the same R-MAT scale 22 graph as the default workload, so the default
    # line can reuse it
    assert spec["graph"] == {k: bench.WORKLOADS["rmat22_s512"][k]
                             for k in ("kind", "scale", "ef", "seed")}
    g = native.wilson_grid(40, 40, 30, 3)
    reqs = bench.make_requests(g, 120, spec["seed"], spec["sizes"])
    assert {int(r.size) for r in reqs} == set(spec["sizes"])


def test_poisson_arrivals_rate():
    assert np.all(bench.poisson_arrivals(5, None, 0) == 0)
    t = bench.poisson_arrivals(20000, 50.0, 3)
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] / 20000 - 1 / 50.0) < 0.05 / 50.0 * 3


def test_latency_summary_small_requests():
    s = bench._latency_summary([1.0, 2.0, 3.0, 100.0], [1, 64, 65, 2048])
    assert s["small_requests"] == 2
    assert s["small_p50_ms"] == 1.5
    assert s["p99_ms"] > 90


def test_level_bytes_model():
    V, W, E = 1000, 16, 8000
    pull = dict(dir=1, active=500, edges=4000, rows=3000, new_vertices=200, new_pairs=900,
                frontier_entries=0, frontier_vertices=0)
    row = 4 * W
    want = 4 * (V + 1) + row * 500 + 4 * 4000 + row * 3000 + 2 * row * 200 + 4 * 900
    assert bench.level_bytes(pull, V, W, E) == want
    push = dict(dir=0, frontier_entries=30, frontier_vertices=20, edges=700, new_vertices=50,
                new_pairs=60, active=0, rows=0)
    want = 8 * 30 + 20 * (8 + row) + 700 * (4 + row) + 50 * (row + 8) + 4 * 60
    assert bench.level_bytes(push, V, W, E) == want
