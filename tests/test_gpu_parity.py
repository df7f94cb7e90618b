"""Bit-exact parity of the sm_103a engine with the CPU oracle (GPU).

Mirrors the reference's GPU suites: golden known answers for every kernel
path (tests/common/oracles.rs), batch sizes straddling word boundaries
(tests/tier2_boundaries/b6_batch_sizes.rs), directed graphs
(tests/tier3_combinations/t3_03_asymmetric_pushpull.rs), duplicate sources,
pooled-buffer re-entrancy (crates/gpu_bfs/tests/m19_adversarial_challenge.rs)
and error behaviour (crates/gpu_bfs/src/engine.rs:228-248). Tolerance: none,
every u32 must match.
"""
import numpy as np
import pytest

from conftest import assert_same, case_graph

pytestmark = pytest.mark.gpu

METHODS = ["Auto", "PushPullAdaptive", "MultiWordBitParallel", "BitParallel64",
           "WorkgroupPersistentBfs", "SparseQueue", "IndirectSparseQueuePush"]


def _oracle(oracle, g, src):
    return oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, src)


@pytest.mark.parametrize("method", METHODS)
def test_golden_cases(native, gpu_engine, golden, method):
    m = native.GpuBfsMethod[method]
    for case in golden["bfs"]:
        g = case_graph(native, case)
        got = gpu_engine.run_ms_bfs_with_method(m, g, case["sources"])
        assert_same(got, case["dist"], g, case["sources"], f"{case['name']}/{method}")


def _graphs(native):
    return {
        "er": native.generate_erdos_renyi_np(3000, 8 / 2999, 1),
        "rmat12": native.generate_graph500_rmat(12, 16, 2),
        "rmat12_directed": native.generate_rmat(12, 8, 0.57, 0.19, 0.19, 0.05, 3, directed=True),
        "tree": native.generate_random_tree(2000, 4),
        "wilson": native.wilson_grid(60, 50, 80, 5),
        "grid64": native.generate_grid2d(64, 64),
        # odd V: per-plane arrays of V*W words start off 16-byte boundaries for W <= 2
        "er_odd": native.generate_erdos_renyi_np(2999, 8 / 2998, 6),
        "tree_odd": native.generate_random_tree(1001, 7),
    }


@pytest.mark.parametrize("S", [1, 3, 17, 31, 33, 63, 65, 129, 512, 700, 2048])
def test_batch_sizes_all_paths(native, gpu_engine, oracle, S):
    rng = np.random.default_rng(S)
    for name, g in _graphs(native).items():
        src = rng.integers(0, g.num_vertices, S).astype(np.uint32)
        want = _oracle(oracle, g, src)
        for method in ("Auto", "PushPullAdaptive", "MultiWordBitParallel", "BitParallel64",
                       "WorkgroupPersistentBfs"):
            got = gpu_engine.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
            assert_same(got, want, g, src, f"{name}/S={S}/{method}")


@pytest.mark.parametrize("max_words", [1, 2, 4, 8, 16, 32, 64])
def test_every_word_width(native, oracle, max_words):
    """Passes of 32*W sources for every compiled W, several passes per call."""
    eng = native.GpuBfsEngine(native.GpuBfsMethod.PushPullAdaptive)
    try:
        eng.set_tuning(max_words_per_pass=max_words)
        g = native.generate_graph500_rmat(11, 8, 11)
        S = 32 * max_words * 2 + 5
        src = np.random.default_rng(max_words).integers(0, g.num_vertices, S).astype(np.uint32)
        want = _oracle(oracle, g, src)
        for method in ("PushPullAdaptive", "MultiWordBitParallel", "BitParallel64"):
            got = eng.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
            assert_same(got, want, g, src, f"W={max_words}/{method}")
        assert eng.last_stats["words_per_vertex"] == max_words
        assert eng.last_stats["passes"] == 3
    finally:
        eng.close()


def test_deep_levels_beyond_level_planes(native, gpu_engine, oracle):
    """Distances >= 256 are written directly (beyond the 8 bit-planes)."""
    g = native.path_graph(1500)
    src = np.array([0, 1499, 700, 3], np.uint32)
    want = _oracle(oracle, g, src)
    for method in ("PushPullAdaptive", "MultiWordBitParallel", "BitParallel64",
                   "WorkgroupPersistentBfs"):
        got = gpu_engine.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
        assert_same(got, want, g, src, f"path1500/{method}")


def test_duplicate_sources_and_isolated(native, gpu_engine, oracle):
    g = native.generate_graph500_rmat(10, 4, 21)
    src = np.array([5, 5, 5, 0, 1023, 5] + list(range(40)), np.uint32)
    want = _oracle(oracle, g, src)
    for method in METHODS:
        got = gpu_engine.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
        assert_same(got, want, g, src, f"dups/{method}")


def test_directed_dag_row(native, gpu_engine, golden):
    case = next(c for c in golden["bfs"] if c["name"] == "dag_50_source_49")
    g = case_graph(native, case)
    src = [0, 10, 20, 30, 40, 49]
    from oracle import oracle as o
    want = o.ms_bfs_fifo(50, g.row_offsets, g.col_indices, src)
    for method in METHODS:
        got = gpu_engine.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
        assert_same(got, want, g, src, f"dag/{method}")
        row = got[5 * 50:6 * 50]
        assert row[49] == 0 and np.all(row[:49] == 0xFFFFFFFF)


def test_errors_match_reference(native, gpu_engine):
    g = native.path_graph(5)
    with pytest.raises(native.BfsError) as ei:
        gpu_engine.run_ms_bfs(g, [1, 2, 7])
    assert ei.value.code == 1
    assert str(ei.value) == "Source vertex 7 at index 2 exceeds graph vertex count 5"
    with pytest.raises(native.BfsError) as ei:
        gpu_engine.run_ms_bfs(native.empty_graph(), [0])
    assert ei.value.code == 2
    assert gpu_engine.run_ms_bfs(g, []).size == 0
    assert gpu_engine.run_ms_bfs(native.empty_graph(), []).size == 0
    m = gpu_engine.run_ms_reachability(native.empty_graph(), [])
    assert m.words.size == 0


def test_pooled_reentrancy_same_shape_graphs(native, gpu_engine, oracle):
    """Two different graphs with identical (V, E) must not share stale state
    (the reference keys its pool on (V, E) only)."""
    a = native.generate_grid2d(40, 40)
    b_edges = [(u, int(v)) for u in range(a.num_vertices)
               for v in a.neighbors((u * 7) % a.num_vertices)]
    b = native.CsrGraph.from_edge_list(a.num_vertices, b_edges)
    src = np.arange(0, 1600, 9, dtype=np.uint32)
    for g in (a, b, a, b):
        for method in ("PushPullAdaptive", "WorkgroupPersistentBfs"):
            got = gpu_engine.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, src)
            assert_same(got, _oracle(oracle, g, src), g, src, f"reentrant/{method}")


def test_reachability(native, gpu_engine, oracle):
    for g, S in ((native.generate_graph500_rmat(11, 8, 31), 700),
                 (native.wilson_grid(30, 30, 20, 2), 65),
                 (native.generate_rmat(10, 8, 0.57, 0.19, 0.19, 0.05, 6, directed=True), 33)):
        src = np.random.default_rng(S).integers(0, g.num_vertices, S).astype(np.uint32)
        dist = _oracle(oracle, g, src)
        want = oracle.reachability_from_distances(g.num_vertices, S, dist)
        got = gpu_engine.run_ms_reachability(g, src)
        assert got.words_per_vertex == (S + 31) // 32
        assert_same(got.words, want, label=f"reach/V={g.num_vertices}/S={S}")


def test_csr_one_shot_entry_and_stats(native, oracle):
    import ctypes as C
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        g = native.generate_graph500_rmat(10, 8, 8)
        src = np.arange(0, 1024, 5, dtype=np.uint32)
        out = np.empty(src.size * g.num_vertices, np.uint32)
        st = native._native.Stats()
        p = native._native.u32p
        rc = native._native.lib().msbfs_run_ms_bfs_csr(
            eng._h, g.num_vertices, g.num_edges, g.row_offsets.ctypes.data_as(p),
            g.col_indices.ctypes.data_as(p), src.ctypes.data_as(p), src.size,
            out.ctypes.data_as(p), C.byref(st))
        assert rc == 0
        want = _oracle(oracle, g, src)
        assert_same(out, want, g, src, "csr one-shot")
        assert st.reached_pairs == int(np.count_nonzero(want != 0xFFFFFFFF))
        assert st.levels >= 2 and st.gpu_ms > 0
    finally:
        eng.close()


def test_device_api_and_traversed_edges(native, gpu_engine, oracle):
    torch = pytest.importorskip("torch")
    g = native.generate_graph500_rmat(12, 16, 41)
    src = native.sample_sources(g, 512, 3, min_degree=1)
    out = torch.empty(src.size * g.num_vertices, dtype=torch.int32, device="cuda")
    gpu_engine.run_ms_bfs_device(g, src, out.data_ptr())
    st = gpu_engine.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    want = _oracle(oracle, g, src)
    assert_same(got, want, g, src, "device api")
    assert st["path"] == 3 and st["pull_levels"] >= 1 and st["push_levels"] >= 1
    te = gpu_engine.traversed_edges_device(g, out.data_ptr(), src.size)
    assert te == oracle.traversed_edges(g.num_vertices, g.row_offsets, src.size, want)


def test_host_loop_fallback(native, oracle, monkeypatch):
    monkeypatch.setenv("MSBFS_HOST_LOOP", "1")
    eng = native.GpuBfsEngine(native.GpuBfsMethod.PushPullAdaptive)
    try:
        g = native.generate_graph500_rmat(11, 8, 13)
        src = np.arange(0, 2048, 3, dtype=np.uint32)
        got = eng.run_ms_bfs(g, src)
        assert_same(got, _oracle(oracle, g, src), g, src, "host loop")
    finally:
        eng.close()


def test_page_locked_host_output(native, oracle):
    """Level-path output written straight into page-locked host memory."""
    torch = pytest.importorskip("torch")
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        for g, S in ((native.generate_graph500_rmat(12, 16, 51), 700),
                     (native.wilson_grid(40, 40, 30, 6), 70)):
            src = np.random.default_rng(S).integers(0, g.num_vertices, S).astype(np.uint32)
            pinned = torch.empty(S * g.num_vertices, dtype=torch.int32, pin_memory=True)
            out = pinned.numpy().view(np.uint32)
            out[:] = 7
            eng.run_ms_bfs_into(g, src, out)
            assert_same(out, _oracle(oracle, g, src), g, src, f"pinned/V={g.num_vertices}")
    finally:
        eng.close()


@pytest.mark.parametrize("mode", ["global", "cluster"])
def test_cta_global_bitmap_beyond_shared_memory(native, oracle, monkeypatch, mode):
    """Road graph whose visited bitmap exceeds shared memory (1,960,000
    vertices > 8 bits x 227 KB). Calls of few sources split the bitmap over
    the shared memory of a thread-block cluster (rank 0 traverses, the other
    ranks' slices are reached through distributed shared memory); otherwise
    (here forced by MSBFS_CTA_CLUSTER=0) each block keeps an L2-resident
    global slab. Rows, statistics and the queue slab that alternates ends by
    level are checked over thousands of levels."""
    monkeypatch.setenv("MSBFS_CTA_CLUSTER", "0" if mode == "global" else "-1")
    g = native.wilson_grid(1400, 1400, 2000, 11)
    src = native.sample_sources(g, 20, 4)
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        got = eng.run_ms_bfs(g, src)
        assert eng.last_stats["path"] == 4  # CTA path, not the level-path fallback
        if mode == "global":
            assert eng.last_stats["cta_cluster"] == 0
        else:
            assert eng.last_stats["cta_cluster"] in (2, 4, 8)
        want = _oracle(oracle, g, src)
        assert_same(got, want, g, src, f"{mode}-bitmap CTA rows")
        st = eng.run_ms_bfs_stats(g, src)
        d = want.reshape(len(src), g.num_vertices).astype(np.int64)
        fin = d != 0xFFFFFFFF
        assert np.array_equal(st["reached"], fin.sum(1))
        assert np.array_equal(st["eccentricity"], np.where(fin, d, 0).max(1))
        assert np.array_equal(st["distance_sum"], np.where(fin, d, 0).sum(1))
    finally:
        eng.close()


def test_cta_cluster_sizes(native, oracle, monkeypatch):
    """Clusters of 2, 4 and 8 blocks: a 9,000,000-vertex grid needs 8 slices
    (1.1 MB of bitmap), a 4,000,000-vertex one 4 (forced even with more
    sources than resident clusters), each with sources in odd slices."""
    monkeypatch.setenv("MSBFS_CTA_CLUSTER", "1")
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        for side, want_cl in ((3000, 8), (2000, 4), (1500, 2)):
            g = native.generate_grid2d(side, side)
            V = g.num_vertices
            src = np.asarray([V - 1, V // 2 + side // 2, 5 * V // 8, 1], np.uint32)
            got = eng.run_ms_bfs(g, src)
            assert eng.last_stats["path"] == 4
            assert eng.last_stats["cta_cluster"] == want_cl
            assert_same(got, _oracle(oracle, g, src), g, src, f"cluster grid {side}")
    finally:
        eng.close()


def test_cta_frontier_beyond_shared_queue(native, oracle):
    """Frontiers larger than the shared-memory queue halves (4,096 entries)
    continue in the global slab: a star (level-1 frontier of 29,999), wide
    random trees and an Erdos-Renyi graph; the 2,000,000-vertex tree runs in
    global-bitmap mode."""
    eng = native.GpuBfsEngine(native.GpuBfsMethod.WorkgroupPersistentBfs)
    try:
        cases = [(native.star_graph(30000), [0, 1, 29999]),
                 (native.generate_random_tree(300000, 9), None),
                 (native.generate_erdos_renyi_np(60000, 8.0 / 59999, 4), None),
                 (native.generate_random_tree(2000000, 10), None),  # global bitmap
                 # road-like grids (edge-record queue entries), sources at the
                 # centre so the diamond-shaped frontiers outgrow the queue
                 # halves: shared bitmap (1,690,000 vertices) and global bitmap
                 (native.generate_grid2d(1300, 1300), [650 * 1300 + 650, 0]),
                 (native.generate_grid2d(3000, 3000), [1500 * 3000 + 1500, 7])]
        for g, src in cases:
            if src is None:
                src = native.sample_sources(g, 9, 2)
            src = np.asarray(src, np.uint32)
            got = eng.run_ms_bfs(g, src)
            assert eng.last_stats["path"] == 4
            assert_same(got, _oracle(oracle, g, src), g, src, f"CTA V={g.num_vertices}")
    finally:
        eng.close()


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_level_cap_times_out_and_engine_recovers(native, oracle, monkeypatch, loop):
    """A pass still running at the level cap stops with MSBFS_ERR_TIMEOUT
    (code 4) through the CUDA-graph WHILE loop and through the host-driven
    loop. Its buffers are left clean -- the frontier it was about to expand
    included -- so a following call on the same workspace (same graph and
    word width) whose traversal ends under the cap is bit-exact. The graph is
    a path of 1,500 vertices (1,499 levels) beside a star of 11 vertices."""
    if loop == "host":
        monkeypatch.setenv("MSBFS_HOST_LOOP", "1")
    edges = [(i, i + 1) for i in range(1499)] + [(1500, 1501 + k) for k in range(10)]
    edges += [(b, a) for a, b in edges]
    g = native.CsrGraph.from_edge_list(1511, edges)
    eng = native.GpuBfsEngine(native.GpuBfsMethod.PushPullAdaptive)
    try:
        deep = np.array([0, 1499, 700, 3], np.uint32)
        star = np.array([1500, 1505, 1501, 1509], np.uint32)
        # Stopped at level 8, the pass leaves level 9's frontier in rotation
        # slot 0, which the next pass's first bottom-up level reads without a
        # frontier-bitmap filter: left uncleared, its path vertices would
        # hand the star's lanes distances on the path.
        eng.set_level_cap(9)
        for method in ("MultiWordBitParallel", "PushPullAdaptive"):
            m = native.GpuBfsMethod[method]
            for _ in range(2):
                with pytest.raises(native.BfsError) as ei:
                    eng.run_ms_bfs_with_method(m, g, deep)
                assert ei.value.code == 4 and "level cap" in str(ei.value)
                assert_same(eng.run_ms_bfs_with_method(m, g, star), _oracle(oracle, g, star),
                            g, star, f"{loop} loop, {method}: same workspace after the cap")
        eng.set_level_cap(0)
        want = _oracle(oracle, g, deep)
        for method in ("PushPullAdaptive", "MultiWordBitParallel", "BitParallel64"):
            got = eng.run_ms_bfs_with_method(native.GpuBfsMethod[method], g, deep)
            assert_same(got, want, g, deep, f"{loop} loop after the cap, {method}")
    finally:
        eng.close()


def test_autotune_same_bytes_and_cache(native, oracle, tmp_path):
    """The level-path autotuner changes speed, never results: rows after
    tuning equal the oracle's; the chosen settings are cached per graph
    class and source bucket, and a fresh engine applies them from the file
    without timing. A road-like graph's calls go to the CTA path and are
    not tuned."""
    cache = str(tmp_path / "level_tuning.txt")
    g = native.generate_graph500_rmat(13, 16, 91)
    src = native.sample_sources(g, 300, 4, min_degree=1)
    want = _oracle(oracle, g, src)
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        t = eng.autotune(g, src, cache_path=cache)
        assert t["level_path"] == 1 and not t["from_cache"] and t["trials"] >= 10
        assert t["class_name"] == "powerlaw/v2^12/s512" and 0 < t["ms"] <= t["default_ms"]
        assert t["max_words_per_pass"] in (4, 8, 16) and t["hub_split"] in (256, 512, 1024)
        assert_same(eng.run_ms_bfs(g, src), want, g, src, f"tuned {t}")
        other = native.sample_sources(g, 260, 5, min_degree=1)  # same bucket, other sources
        assert_same(eng.run_ms_bfs(g, other), _oracle(oracle, g, other), g, other, "tuned, other")
    finally:
        eng.close()
    eng = native.GpuBfsEngine(native.GpuBfsMethod.Auto)
    try:
        t2 = eng.autotune(g, src, cache_path=cache)
        assert t2["from_cache"] and t2["trials"] == 0
        keys = ("max_words_per_pass", "alpha", "beta", "hub_split", "bitmap_div",
                "warp_scan_degree")
        assert {k: t2[k] for k in keys} == {k: t[k] for k in keys}
        assert_same(eng.run_ms_bfs(g, src), want, g, src, "settings from the cache")
        road = native.wilson_grid(50, 50, 40, 2)
        rs = native.sample_sources(road, 40, 1)
        assert eng.autotune(road, rs)["level_path"] == 0
        assert len(open(cache).read().splitlines()) == 1
    finally:
        eng.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_byte_row_transport_mixed_passes(native, oracle, monkeypatch, pinned):
    """Rows bound for pageable host memory travel as one byte per distance
    when every distance of a pass is below 255 and are widened on the host;
    deeper passes keep u32 rows (page-locked output always gets u32 rows
    written over the link). A graph of an R-MAT component beside a path of
    400 vertices, with passes of 32 sources: the first pass's sources sit
    in the R-MAT part (byte rows), the second's include the path's end
    (levels up to 399, u32 rows). Rows equal the oracle's and those of an
    engine that never narrows (MSBFS_NARROW=0), for pageable and
    page-locked output."""
    torch = pytest.importorskip("torch")
    r = native.generate_graph500_rmat(10, 8, 17)
    n0 = r.num_vertices
    edges = [(u, int(v)) for u in range(n0) for v in r.neighbors(u)]
    edges += [(n0 + i, n0 + i + 1) for i in range(399)]
    edges += [(n0 + i + 1, n0 + i) for i in range(399)]
    g = native.CsrGraph.from_edge_list(n0 + 400, edges)
    deg = np.diff(r.row_offsets.astype(np.int64))
    live = np.flatnonzero(deg > 0).astype(np.uint32)
    src = np.concatenate([live[:32], live[32:60], np.array([n0, n0 + 399, n0 + 7, n0 + 200],
                                                           np.uint32)]).astype(np.uint32)
    want = _oracle(oracle, g, src)
    outs = {}
    for narrow in ("1", "0"):
        monkeypatch.setenv("MSBFS_NARROW", narrow)
        eng = native.GpuBfsEngine(native.GpuBfsMethod.PushPullAdaptive)
        try:
            eng.set_tuning(max_words_per_pass=1)
            if pinned:
                buf = torch.empty(src.size * g.num_vertices, dtype=torch.int32, pin_memory=True)
                out = buf.numpy().view(np.uint32)
                out[:] = 7
                eng.run_ms_bfs_into(g, src, out)
                out = out.copy()
            else:
                out = eng.run_ms_bfs(g, src)
            assert eng.last_stats["passes"] == 2 and eng.last_stats["levels"] >= 399
        finally:
            eng.close()
        assert_same(out, want, g, src, f"narrow={narrow} pinned={pinned}")
        outs[narrow] = out
    assert np.array_equal(outs["1"], outs["0"])


@pytest.mark.parametrize("depth", [7, 8, 127, 128, 200, 254, 255, 256])
def test_materialisation_depth_boundaries(native, oracle, monkeypatch, depth):
    """Distances come out of the level planes by a bit-matrix transpose when
    every distance is below 255 (sign-replicating byte selects up to 7 planes,
    a compare at 8) and by per-plane bit extraction otherwise. An R-MAT
    component beside a path of depth + 1 vertices (odd and even vertex
    counts), sources including the path's end so the deepest distance is
    `depth`: u32 rows (never narrowed), byte rows widened on the host, and
    page-locked output, at one and at several words per vertex, all equal
    the oracle's."""
    torch = pytest.importorskip("torch")
    r = native.generate_graph500_rmat(10, 8, 23)
    n0 = r.num_vertices
    edges = [(u, int(v)) for u in range(n0) for v in r.neighbors(u)]
    edges += [(n0 + i, n0 + i + 1) for i in range(depth)]
    edges += [(n0 + i + 1, n0 + i) for i in range(depth)]
    g = native.CsrGraph.from_edge_list(n0 + depth + 1, edges)
    deg = np.diff(r.row_offsets.astype(np.int64))
    live = np.flatnonzero(deg > 0).astype(np.uint32)
    src = np.concatenate([live[:37], np.array([n0 + depth, n0 + depth // 2, n0], np.uint32)])
    want = _oracle(oracle, g, src)
    for narrow, pinned in (("0", False), ("1", False), ("1", True)):
        monkeypatch.setenv("MSBFS_NARROW", narrow)
        for words in (1, 16):
            eng = native.GpuBfsEngine(native.GpuBfsMethod.PushPullAdaptive)
            try:
                eng.set_tuning(max_words_per_pass=words)
                if pinned:
                    buf = torch.empty(src.size * g.num_vertices, dtype=torch.int32,
                                      pin_memory=True)
                    out = buf.numpy().view(np.uint32)
                    out[:] = 7
                    eng.run_ms_bfs_into(g, src, out)
                    out = out.copy()
                else:
                    out = eng.run_ms_bfs(g, src)
                assert eng.last_stats["levels"] >= depth
            finally:
                eng.close()
            assert_same(out, want, g, src, f"depth={depth} narrow={narrow} pinned={pinned} W={words}")
