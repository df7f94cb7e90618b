"""Batched form: many graphs in one persistent launch, autotuned per graph
class, bit-exact against the CPU oracle and against the plain per-graph path
(GPU)."""
import numpy as np
import pytest

from conftest import assert_same

pytestmark = pytest.mark.gpu


def _mixed_batch(native, n_er=10, n_grid=6, n_rmat=4, seed=0):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n_er):
        n = int(np.exp(rng.uniform(np.log(200), np.log(4000))))
        items.append(native.generate_erdos_renyi_np(n, 8 / (n - 1), 100 + i))
    for i in range(n_grid):
        k = int(rng.integers(8, 48))
        items.append(native.wilson_grid(k, k, max(1, k * k // 50), 200 + i))
    for i in range(n_rmat):
        items.append(native.generate_graph500_rmat(11, 8, 300 + i))
    items.append(native.generate_rmat(10, 8, 0.57, 0.19, 0.19, 0.05, 7, directed=True))
    items.append(native.path_graph(700))
    out = []
    for g in items:
        S = int(np.exp(rng.uniform(0, np.log(256))))
        src = rng.integers(0, g.num_vertices, S).astype(np.uint32)
        out.append((g, src))
    return out


def test_batched_matches_oracle_and_plain(native, oracle, tmp_path):
    items = _mixed_batch(native)
    b = native.BatchedBfs(items)
    try:
        cache = str(tmp_path / "tune.txt")
        b.autotune(samples_per_class=2, cache_path=cache)
        ms = b.run()
        assert ms > 0
        want = [oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, s)
                for g, s in items]
        for i, (g, s) in enumerate(items):
            assert_same(b.result(i), want[i], g, s, f"batched graph {i} {b.config(i)}")
        # the plain path writes the same buffers
        b.run_per_graph()
        for i, (g, s) in enumerate(items):
            assert_same(b.result(i), want[i], g, s, f"per-graph {i}")
        # cached configurations are reused by a fresh batch
        b2 = native.BatchedBfs(items[:5])
        b2.autotune(samples_per_class=2, cache_path=cache)
        assert b2.config(0) == b.config(0)
        b2.run()
        for i in range(5):
            g, s = items[i]
            assert_same(b2.result(i), want[i], g, s, f"cached config {i}")
        b2.close()
    finally:
        b.close()


@pytest.mark.parametrize("alg_case", ["untuned", "every_class_each_candidate"])
def test_batched_untuned_and_rerun(native, oracle, alg_case):
    items = _mixed_batch(native, n_er=4, n_grid=3, n_rmat=2, seed=5)
    b = native.BatchedBfs(items)
    try:
        if alg_case != "untuned":
            b.autotune(samples_per_class=1)
        for _ in range(2):  # reruns reuse the per-block scratch
            b.run()
            for i, (g, s) in enumerate(items):
                want = oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, s)
                assert_same(b.result(i), want, g, s, f"{alg_case} {i}")
    finally:
        b.close()


@pytest.mark.parametrize("div", [2, 1024])
def test_batched_vertex_tiles_match_oracle(native, oracle, tmp_path, div):
    """The vertex-tile shape (a thread per vertex holding all its words),
    forced for every class through the autotuner's cache file, with a
    bottom-up threshold that makes nearly every level bottom-up (div 2 is
    for graphs whose frontier exceeds V/2; 1024 sends almost every level
    bottom-up) -- rows equal the oracle's at 2, 4 and 8 words per vertex."""
    items = _mixed_batch(native, n_er=6, n_grid=3, n_rmat=3, seed=9)
    b = native.BatchedBfs(items)
    try:
        classes = sorted({b.config(i)["class"] for i in range(len(items))})
    finally:
        b.close()
    for words in (2, 4, 8):
        cache = tmp_path / f"vertex_tiles_{words}_{div}.txt"
        # "class alg wcap div chunk shape ms": bit-parallel, vertex tiles
        cache.write_text("".join(f"{c} 0 {words} {div} 4 1 1.0\n" for c in classes))
        b = native.BatchedBfs(items)
        try:
            b.autotune(samples_per_class=1, cache_path=str(cache))
            assert all(b.config(i)["alg"] == "bit_parallel_vertex_tiles"
                       for i in range(len(items)))
            b.run()
            for i, (g, s) in enumerate(items):
                want = oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, s)
                assert_same(b.result(i), want, g, s, f"vertex tiles W<={words} div={div} {i}")
        finally:
            b.close()
