"""Per-source reductions and the served form (GPU).

The served form packs unrelated requests into the source lanes of shared
traversals; each request's result must be the same bytes alone and in the
mix, and equal to the CPU oracle.
"""
import threading

import numpy as np
import pytest

from conftest import assert_same

pytestmark = pytest.mark.gpu

MAX = 0xFFFFFFFF


def _oracle_stats(oracle, g, src):
    d = oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, src)
    d = d.reshape(len(src), g.num_vertices).astype(np.int64)
    fin = d != MAX
    out = np.zeros(len(src), [("distance_sum", "<u8"), ("eccentricity", "<u4"),
                              ("reached", "<u4")])
    out["distance_sum"] = np.where(fin, d, 0).sum(1)
    out["eccentricity"] = np.where(fin, d, 0).max(1)
    out["reached"] = fin.sum(1)
    return out


def _same_stats(got, want, label):
    for f in ("distance_sum", "eccentricity", "reached"):
        assert np.array_equal(got[f], want[f]), f"{label}: field {f} differs"


@pytest.mark.parametrize("method", ["Auto", "PushPullAdaptive", "MultiWordBitParallel",
                                    "WorkgroupPersistentBfs"])
def test_source_stats_match_oracle(native, oracle, method):
    eng = native.GpuBfsEngine(native.GpuBfsMethod[method])
    try:
        cases = [(native.generate_graph500_rmat(12, 16, 61), 700),
                 (native.wilson_grid(50, 40, 40, 7), 300),
                 (native.path_graph(1500), 5),  # levels beyond the 8 planes
                 (native.generate_rmat(10, 8, 0.57, 0.19, 0.19, 0.05, 8, directed=True), 40),
                 # several vertex chunks, the last one ragged; 2- and 4-word passes
                 (native.wilson_grid(71, 73, 40, 9), 33),
                 (native.generate_graph500_rmat(13, 8, 62), 100)]
        for g, S in cases:
            src = np.random.default_rng(S).integers(0, g.num_vertices, S).astype(np.uint32)
            got = eng.run_ms_bfs_stats(g, src)
            _same_stats(got, _oracle_stats(oracle, g, src), f"{method} V={g.num_vertices}")
    finally:
        eng.close()


def _requests(rng, V, n):
    sizes = [1, 8, 64, 512, 2048]
    out = []
    for i in range(n):
        S = sizes[int(rng.integers(0, len(sizes)))]
        mode = int(rng.integers(0, 2))
        out.append((rng.integers(0, V, S).astype(np.uint32), mode))
    return out


@pytest.mark.parametrize("graph_kind,express,lanes", [("rmat", 0, 512), ("road", 0, 512),
                                                      ("rmat", 1, 512), ("road", 1, 512),
                                                      ("rmat", 1, 2048)])
def test_server_mix_equals_alone_equals_oracle(native, oracle, graph_kind, express, lanes):
    """Mixed requests from two threads equal the same requests alone and the
    oracle. With 2,048 lanes per launch the general slots run each launch as
    one pass of up to 64 words per vertex."""
    torch = pytest.importorskip("torch")
    if graph_kind == "rmat":
        g = native.generate_graph500_rmat(12, 8, 71)
    else:
        g = native.wilson_grid(60, 60, 72, 8)
    V = g.num_vertices
    rng = np.random.default_rng(3 + express)
    reqs = _requests(rng, V, 14)
    slots = 2 + express
    srv = native.BfsServer(g, slots=slots, max_sources_per_launch=lanes,
                           hbm_budget_bytes=slots * 300 * V * 4,  # forces row splitting
                           express_slots=express, small_sources=8,
                           general_sm_percent=70 if express else 100)
    try:
        # in the mix: submitted from two threads, interleaved
        tickets = [None] * len(reqs)

        def client(idx):
            for i in idx:
                src, mode = reqs[i]
                out = None
                if mode == srv.ROWS and i % 3 == 0:  # some outputs page-locked
                    out = torch.empty(src.size * V, dtype=torch.int32,
                                      pin_memory=True).numpy().view(np.uint32)
                tickets[i] = srv.submit(src, mode, out)

        th = [threading.Thread(target=client, args=(list(range(k, len(reqs), 2)),))
              for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        mixed = []
        for i, t in enumerate(tickets):
            res, info = srv.wait(t)
            assert info["status"] == 0 and info["latency_ms"] >= info["queue_ms"] >= 0
            mixed.append(res.copy())
        # alone: one request at a time through the same server
        for i, (src, mode) in enumerate(reqs):
            res, _ = srv.wait(srv.submit(src, mode))
            if mode == srv.ROWS:
                assert_same(res, mixed[i], g, src, f"request {i} alone vs mix")
                want = oracle.ms_bfs_fifo(V, g.row_offsets, g.col_indices, src)
                assert_same(res, want, g, src, f"request {i} vs oracle")
            else:
                assert res.tobytes() == mixed[i].tobytes(), f"request {i} stats alone vs mix"
                _same_stats(res, _oracle_stats(oracle, g, src), f"request {i} stats")
        c = srv.counters()
        assert c["traversals"] >= 1 and c["kernel_launches"] >= c["traversals"]
    finally:
        srv.close()


def test_server_config_rejected(native):
    g = native.generate_graph500_rmat(8, 8, 5)
    with pytest.raises(native.BfsError):
        native.BfsServer(g, slots=2, express_slots=2)  # no general slot left
    with pytest.raises(native.BfsError):
        native.BfsServer(g, slots=2, general_sm_percent=101)


def test_sm_share_same_results(native, oracle):
    g = native.generate_graph500_rmat(12, 16, 77)
    src = native.sample_sources(g, 300, 5, min_degree=1)
    eng = native.GpuBfsEngine()
    try:
        full = eng.run_ms_bfs(g, src)
        for pct in (1, 37):
            eng.set_sm_share(pct)
            assert_same(eng.run_ms_bfs(g, src), full, g, src, f"sm share {pct}%")
        with pytest.raises(native.BfsError):
            eng.set_sm_share(0)
        road = native.wilson_grid(40, 40, 30, 3)  # CTA path
        rs = native.sample_sources(road, 50, 1)
        assert_same(eng.run_ms_bfs(road, rs),
                    oracle.ms_bfs_fifo(road.num_vertices, road.row_offsets, road.col_indices,
                                       rs), road, rs, "CTA path, sm share 37%")
    finally:
        eng.close()


def test_server_wait_timeout_and_empty(native, oracle):
    """A wait whose limit runs out returns MSBFS_ERR_TIMEOUT (code 4) and
    keeps the ticket; a later wait returns the result. The request (2,048
    distance rows on a road graph of ~1,000 levels) takes milliseconds, the
    first wait's limit is 10 microseconds."""
    g = native.wilson_grid(339, 338, 5000, 1442)
    srv = native.BfsServer(g, slots=1)
    try:
        t = srv.submit(np.zeros(0, np.uint32), srv.STATS)
        res, info = srv.wait(t)
        assert res.size == 0 and info["launches"] == 0
        with pytest.raises(native.BfsError):
            srv.submit(np.array([g.num_vertices], np.uint32), srv.STATS)
        src = native.sample_sources(g, 2048, 7)
        t = srv.submit(src, srv.ROWS)
        with pytest.raises(native.BfsError) as ei:
            srv.wait(t, timeout_ms=0.01)
        assert ei.value.code == 4
        res, info = srv.wait(t)
        assert info["status"] == 0 and info["latency_ms"] > 0.01
        want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, src)
        assert_same(res, want, g, src, "rows after an expired wait")
    finally:
        srv.close()


def test_server_admits_row_launches_by_free_pool_bytes(native, oracle):
    """Distance rows are staged in one pool shared by the slots: a launch
    takes only as many lanes as the largest free range holds rows for. With
    a pool of 40 lanes' rows and three slots, concurrent row requests of up
    to 200 sources are cut into launches of at most 40 lanes, and every
    result is still the oracle's."""
    g = native.generate_graph500_rmat(11, 8, 81)
    V = g.num_vertices
    srv = native.BfsServer(g, slots=3, max_sources_per_launch=512, hbm_budget_bytes=40 * V * 4)
    try:
        rng = np.random.default_rng(12)
        reqs = [rng.integers(0, V, S).astype(np.uint32) for S in (200, 7, 64, 1, 150, 33)]
        tickets = [srv.submit(r, srv.ROWS) for r in reqs]
        for r, t in zip(reqs, tickets):
            res, info = srv.wait(t)
            assert info["status"] == 0
            assert info["launches"] >= -(-r.size // 40)
            assert_same(res, oracle.ms_bfs_fifo(V, g.row_offsets, g.col_indices, r), g, r,
                        f"{r.size} sources through a 40-lane pool")
        # statistics need no rows: a request of 300 sources is one launch
        src = rng.integers(0, V, 300).astype(np.uint32)
        res, info = srv.wait(srv.submit(src, srv.STATS))
        assert info["launches"] == 1
    finally:
        srv.close()
