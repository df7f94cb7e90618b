"""Host graph core of libmsbfs.so vs the reference's literals and the oracle
(no GPU: these entry points run on the host)."""
import numpy as np
import pytest

from conftest import assert_same


def test_csr_literals(native, golden):
    core = golden["core"]
    c = core["csr_construction"]
    g = native.CsrGraph.from_edge_list(c["num_vertices"], c["edges"])
    assert g.row_offsets.tolist() == c["row_offsets"]
    assert g.col_indices.tolist() == c["col_indices"]
    assert g.max_degree() == c["max_degree"]
    assert [g.degree(u) for u in range(3)] == [2, 1, 1]
    g.validate()
    c = core["self_loops_and_duplicates"]
    g = native.CsrGraph.from_edge_list(c["num_vertices"], c["edges"])
    assert g.row_offsets.tolist() == c["row_offsets"]
    assert g.col_indices.tolist() == c["col_indices"]
    c = core["transpose"]
    g = native.CsrGraph.from_edge_list(c["num_vertices"], c["edges"])
    csc = g.to_csc()
    assert csc.col_offsets.tolist() == c["col_offsets"]
    assert csc.row_indices.tolist() == c["row_indices"]
    assert [csc.in_degree(v) for v in range(3)] == [0, 1, 2]
    assert csc.to_csr() == g
    c = core["symmetry"]
    assert not native.CsrGraph.from_edge_list(3, c["asymmetric"]).is_symmetric()
    assert native.CsrGraph.from_edge_list(3, c["symmetric"]).is_symmetric()
    c = core["to_undirected"]
    u = native.CsrGraph.from_edge_list(3, c["edges"]).to_undirected()
    assert u.row_offsets.tolist() == c["row_offsets"]
    assert u.col_indices.tolist() == c["col_indices"]
    assert u.is_symmetric()


def test_grid_generator_matches_reference_layout(native, golden):
    c = golden["core"]["grid_4x3_csr"]
    g = native.generate_grid2d(c["width"], c["height"])
    assert g.num_edges == c["num_edges"]
    assert g.row_offsets.tolist() == c["row_offsets"]
    assert g.col_indices.tolist() == c["col_indices"]
    for case in golden["bfs"]:
        if case["name"].startswith("grid_"):
            w, h = map(int, case["name"].split("_")[1].split("x"))
            gg = native.generate_grid2d(w, h)
            assert gg.row_offsets.tolist() == case["row_offsets"]
            assert gg.col_indices.tolist() == case["col_indices"]


def test_topology_generators_match_golden(native, golden):
    by = {c["name"]: c for c in golden["bfs"]}
    for name, g in [("path_50_s1", native.path_graph(50)), ("cycle_60_s1", native.cycle_graph(60)),
                    ("star_200_s3", native.star_graph(200)),
                    ("disconnected_cliques_5_7_3", native.disconnected_cliques([5, 7, 3]))]:
        assert g.row_offsets.tolist() == by[name]["row_offsets"], name
        assert g.col_indices.tolist() == by[name]["col_indices"], name


def test_reachability_bitmask_literal(native, golden):
    c = golden["core"]["reachability_bitmask"]
    V, S = c["num_vertices"], c["num_sources"]
    m = native.ReachabilityBitmask.zeroed(V, S)
    assert m.words_per_vertex == 3 and m.words.size == 15
    for s, v, _ in c["finite"]:
        m.set_reachable(s, v)
    assert m.words.tolist() == c["words"]
    assert m.is_reachable(33, 0) and not m.is_reachable(32, 0)
    assert m.reachable_source_count(0) == 2 and m.total_reachable_pairs() == 3
    dist = np.full(S * V, 0xFFFFFFFF, np.uint32)
    for s, v, d in c["finite"]:
        dist[s * V + v] = d
    assert native.ReachabilityBitmask.from_canonical_distances(V, S, dist) == m


@pytest.mark.parametrize("seed", range(4))
def test_edge_list_and_transpose_vs_oracle(native, oracle, seed):
    rng = np.random.default_rng(100 + seed)
    V = int(rng.integers(1, 3000))
    e = rng.integers(0, V, size=(int(rng.integers(0, 8 * V)), 2))
    g = native.CsrGraph.from_edge_list(V, e)
    ro, ci = oracle.csr_from_edge_list(V, e)
    assert_same(g.row_offsets, ro, label="row_offsets")
    assert_same(g.col_indices, ci, label="col_indices")
    csc = g.to_csc()
    co, ri = oracle.to_csc(V, ro, ci)
    assert_same(csc.col_offsets, co, label="col_offsets")
    assert_same(csc.row_indices, ri, label="row_indices")
    assert g.is_symmetric() == oracle.is_symmetric(V, ro, ci)
    u = g.to_undirected()
    assert u.is_symmetric()
    ro2, ci2 = oracle.csr_from_edge_list(V, np.concatenate([e, e[:, ::-1]]))
    assert_same(u.col_indices, ci2, label="undirected")


def test_validate_rejects_malformed(native):
    bad = [
        native.CsrGraph(3, [1, 1, 1, 1], []),           # nonzero start
        native.CsrGraph(3, [0, 2, 1, 2], [1, 2]),       # non-monotonic
        native.CsrGraph(2, [0, 1, 2], [1, 5]),          # column out of bounds
        native.CsrGraph(3, [0, 2, 2, 2], [2, 1]),       # unsorted
        native.CsrGraph(3, [0, 2, 2, 2], [1, 1]),       # duplicate
    ]
    for g in bad:
        with pytest.raises(native.BfsError):
            g.validate()


@pytest.mark.parametrize("maker", [
    lambda m: m.generate_erdos_renyi_np(500, 0.02, 1),
    lambda m: m.generate_random_tree(300, 2),
    lambda m: m.generate_graph500_rmat(9, 8, 3),
    lambda m: m.wilson_grid(40, 30, 60, 4),
    lambda m: m.generate_rmat(8, 4, 0.57, 0.19, 0.19, 0.05, 5, directed=True),
])
def test_generator_invariants(native, maker):
    """generators.rs:666-741: validate, symmetric (undirected), tree edge counts."""
    g = maker(native)
    g.validate()
    assert np.all(g.col_indices < g.num_vertices)


def test_generator_specifics(native, oracle):
    t = native.generate_random_tree(100, 42)
    assert t.num_edges == 2 * 99 and t.is_symmetric()
    d = oracle.ms_bfs_fifo(100, t.row_offsets, t.col_indices, [0])
    assert np.all(d != 0xFFFFFFFF), "random tree must be connected"
    w = native.wilson_grid(339, 338, 5000, 2)
    assert w.num_vertices == 114582 and w.is_symmetric()
    assert w.num_edges == 2 * (114581 + 5000)
    assert w.max_degree() <= 4
    d = oracle.ms_bfs_fifo(w.num_vertices, w.row_offsets, w.col_indices, [0])
    assert np.all(d != 0xFFFFFFFF), "spanning tree + extras is connected"
    r = native.generate_graph500_rmat(10, 16, 9)
    r2 = native.generate_graph500_rmat(10, 16, 9)
    assert r == r2, "seeded generator is deterministic"
    assert r.is_symmetric() and r.num_vertices == 1024
    src = native.sample_sources(r, 64, 5, min_degree=1)
    assert np.all(np.diff(src.astype(np.int64)) > 0)
    assert np.all(r.degrees()[src] >= 1)
    er = native.generate_erdos_renyi_np(2000, 8 / 1999, 11)
    assert er.is_symmetric()
    assert 6.0 < er.avg_degree() < 10.0
