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


class _PlantedOracle:
    """The oracle with one wrong distance planted in the rows it returns (the
    comparison must report exactly that value)."""

    def __init__(self, oracle, row, vertex):
        self._o, self.row, self.vertex = oracle, row, vertex
        self.planted = False

    def ms_bfs_threaded(self, V, ro, ci, src, threads=0):
        d = self._o.ms_bfs_threaded(V, ro, ci, src, threads).copy()
        if not self.planted and self.row < len(src):  # first call only
            d[self.row * V + self.vertex] ^= 1
            self.planted = True
        return d

    def ms_bfs_fifo(self, V, ro, ci, src):
        return self._o.ms_bfs_fifo(V, ro, ci, src)


def test_cpu_sample_rate_compares_every_sampled_row(native, oracle):
    g = native.generate_graph500_rmat(9, 8, 4)
    src = native.sample_sources(g, 40, 2, min_degree=1)
    V = g.num_vertices
    truth = oracle.ms_bfs_fifo(V, g.row_offsets, g.col_indices, src)

    def gpu_rows(i0, i1):
        return [truth[i0 * V:i1 * V], truth[i0 * V:i1 * V].copy()]

    rate, n, threads, secs, parity = bench.cpu_sample_rate(oracle, g, src, target_s=60.0,
                                                           gpu_rows=gpu_rows)
    assert n == 40 and rate > 0 and secs > 0
    assert parity["rows_compared"] == 40 and parity["mismatches"] == 0
    assert not bench.parity_failed({"parity": parity})
    planted = _PlantedOracle(oracle, 3, 17)
    _, _, _, _, parity = bench.cpu_sample_rate(planted, g, src, target_s=60.0,
                                               gpu_rows=gpu_rows)
    # the one planted value differs from both compared outputs
    assert parity["mismatches"] == 2 and parity["mismatched_rows"] == 2
    assert parity["first_mismatch"]["vertex"] == 17
    assert bench.parity_failed({"forms": {"x": {"parity": parity}}})


def test_fifo_single_rate(native, oracle):
    g = native.wilson_grid(30, 30, 20, 1)
    rate, n, secs = bench.cpu_fifo_single(oracle, g, np.arange(10, dtype=np.uint32),
                                          target_s=0.0)
    assert n == 1 and rate > 0 and secs > 0


def test_served_parity_counts_planted_mistake(native, oracle):
    g = native.wilson_grid(30, 20, 15, 2)
    reqs = bench.make_requests(g, 6, 9, sizes=(1, 8))
    outs = []
    for r in reqs:
        ecc, reached, dsum = bench.oracle_stats(oracle, g, r)
        o = np.zeros(r.size, native.SOURCE_STATS_DTYPE)
        o["eccentricity"], o["reached"], o["distance_sum"] = ecc, reached, dsum
        outs.append(o)
    p = bench.served_parity(oracle, g, reqs, outs, 1000)
    assert p["requests_compared"] == 6 and p["mismatches"] == 0
    # a wrong distance in the oracle's rows of the first request changes its
    # distance sum (and possibly its eccentricity)
    p = bench.served_parity(_PlantedOracle(oracle, 0, int(reqs[0][0]) ^ 1), g, reqs, outs, 1000)
    assert p["mismatches"] >= 1


def test_both_arms_print_the_same_config(native):
    g = native.wilson_grid(30, 30, 20, 1)
    spec = dict(kind="road", w=30, h=30, extra=20, S=256, seed=1)
    a = bench.workload_config("road_s256", spec, g)
    b = bench.workload_config("road_s256", spec, g)
    assert a == b and "l2_policy" in a and a["sources"] == 256
