"""CPU oracle pinned against the reference's known answers (no GPU).

The oracle restates crates/cpu_bfs (FIFO, Rayon, bit-parallel-64) and the
CSR helpers of crates/core/src/graph.rs. Each golden case is a closed-form
known answer from the reference's own tests (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import assert_same

MAX = 0xFFFFFFFF


def _algos(oracle):
    return {
        "fifo": oracle.ms_bfs_fifo,
        "threaded": lambda V, ro, ci, s: oracle.ms_bfs_threaded(V, ro, ci, s, threads=4),
        "bit_parallel": oracle.ms_bfs_bit_parallel,
    }


def test_golden_bfs_cases_all_oracle_paths(oracle, golden):
    for case in golden["bfs"]:
        V = case["num_vertices"]
        for name, fn in _algos(oracle).items():
            got = fn(V, case["row_offsets"], case["col_indices"], case["sources"])
            assert_same(got, case["dist"], label=f"{case['name']}/{name}")


def test_golden_symmetry_flags(oracle, golden):
    for case in golden["bfs"]:
        if "symmetric" in case:
            assert oracle.is_symmetric(case["num_vertices"], case["row_offsets"],
                                       case["col_indices"]) == case["symmetric"], case["name"]


def test_csr_literals(oracle, golden):
    core = golden["core"]
    c = core["csr_construction"]
    ro, ci = oracle.csr_from_edge_list(c["num_vertices"], c["edges"])
    assert ro.tolist() == c["row_offsets"] and ci.tolist() == c["col_indices"]
    c = core["self_loops_and_duplicates"]
    ro, ci = oracle.csr_from_edge_list(c["num_vertices"], c["edges"])
    assert ro.tolist() == c["row_offsets"] and ci.tolist() == c["col_indices"]
    c = core["transpose"]
    ro, ci = oracle.csr_from_edge_list(c["num_vertices"], c["edges"])
    co, ri = oracle.to_csc(c["num_vertices"], ro, ci)
    assert co.tolist() == c["col_offsets"] and ri.tolist() == c["row_indices"]
    # round trip (graph.rs:712-714)
    ro2, ci2 = oracle.to_csc(c["num_vertices"], co, ri)
    assert ro2.tolist() == ro.tolist() and ci2.tolist() == ci.tolist()
    c = core["symmetry"]
    ro, ci = oracle.csr_from_edge_list(3, c["asymmetric"])
    assert not oracle.is_symmetric(3, ro, ci)
    ro, ci = oracle.csr_from_edge_list(3, c["symmetric"])
    assert oracle.is_symmetric(3, ro, ci)


def test_reachability_literal(oracle, golden):
    c = golden["core"]["reachability_bitmask"]
    V, S = c["num_vertices"], c["num_sources"]
    dist = np.full(S * V, MAX, np.uint32)
    for s, v, d in c["finite"]:
        dist[s * V + v] = d
    words = oracle.reachability_from_distances(V, S, dist)
    assert words.tolist() == c["words"]


def test_source_validation_matches_reference_message(oracle):
    with pytest.raises(oracle.SourceOutOfBounds) as ei:
        oracle.ms_bfs_fifo(5, [0, 0, 0, 0, 0, 0], [], [1, 2, 7])
    assert str(ei.value) == "Source vertex 7 at index 2 exceeds graph vertex count 5"


def test_empty_inputs(oracle):
    assert oracle.ms_bfs_fifo(0, [0], [], [0]).size == 0
    assert oracle.ms_bfs_fifo(4, [0, 0, 0, 0, 0], [], []).size == 0


def _random_csr(rng, V, m, directed):
    u = rng.integers(0, V, m)
    v = rng.integers(0, V, m)
    e = np.stack([u, v], 1)
    if not directed:
        e = np.concatenate([e, e[:, ::-1]])
    return e


@pytest.mark.parametrize("seed", range(6))
def test_three_way_equivalence_random(oracle, seed):
    """crates/cpu_bfs/src/tests.rs:13-31: FIFO == Rayon == BitParallel."""
    rng = np.random.default_rng(seed)
    V = int(rng.integers(1, 400))
    m = int(rng.integers(0, 4 * V))
    e = _random_csr(rng, V, m, directed=bool(seed % 2))
    ro, ci = oracle.csr_from_edge_list(V, e)
    S = int(rng.integers(1, 140))
    src = rng.integers(0, V, S)
    a = oracle.ms_bfs_fifo(V, ro, ci, src)
    b = oracle.ms_bfs_threaded(V, ro, ci, src, threads=3)
    c = oracle.ms_bfs_bit_parallel(V, ro, ci, src)
    assert_same(b, a, label="threaded")
    assert_same(c, a, label="bit_parallel")
    # metric axioms (tests/common/oracles.rs:45-103)
    d = a.reshape(S, V).astype(np.int64)
    for si, s in enumerate(src):
        assert d[si, s] == 0
    us = np.repeat(np.arange(V), np.diff(ro))
    for si in range(S):
        du, dv = d[si, us], d[si, ci]
        fin = du != MAX
        assert np.all(dv[fin] <= du[fin] + 1)
