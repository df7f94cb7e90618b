"""Generates tests/golden/known_answers.json.

Every case restates a known-answer test of the reference (likr-sandbox/
webgpu-bfs) in closed form: the expected values come from the formulas and
literals those tests assert, never from a BFS. The reference is Rust and
cannot run here, so its tests' literals and analytic oracles are the golden
vectors that pin the CPU oracle (oracle/oracle.c) and, through it, the engine.

Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
from pathlib import Path

MAX = 0xFFFFFFFF
OUT = Path(__file__).resolve().parent / "known_answers.json"


def grid_csr(w: int, h: int):
    """Grid2D::new neighbour order N, W, E, S (crates/core/src/generators.rs:28-80)."""
    ro, ci = [0], []
    for y in range(h):
        for x in range(w):
            v = y * w + x
            if y > 0:
                ci.append(v - w)
            if x > 0:
                ci.append(v - 1)
            if x + 1 < w:
                ci.append(v + 1)
            if y + 1 < h:
                ci.append(v + w)
            ro.append(len(ci))
    return ro, ci


def manhattan(w: int, sources, V: int):
    """Grid2D::ms_bfs_oracle (generators.rs:110-127): |dx| + |dy|."""
    out = []
    for s in sources:
        sx, sy = s % w, s // w
        out += [abs(v % w - sx) + abs(v // w - sy) for v in range(V)]
    return out


def edges_to_csr(V: int, edges):
    """CsrGraph::from_edge_list rules (graph.rs:51-79) for tiny literal graphs."""
    es = sorted({(u, v) for u, v in edges if u != v and u < V and v < V})
    ro = [0] * (V + 1)
    for u, _ in es:
        ro[u + 1] += 1
    for i in range(V):
        ro[i + 1] += ro[i]
    return ro, [v for _, v in es]


def path_csr(n: int):
    """path_graph (generators.rs:392-418)."""
    ro, ci = [0], []
    for u in range(n):
        if u > 0:
            ci.append(u - 1)
        if u + 1 < n:
            ci.append(u + 1)
        ro.append(len(ci))
    return ro, ci


def cycle_csr(n: int):
    """cycle_graph (generators.rs:452-482): sorted (prev, next)."""
    ro, ci = [0], []
    for u in range(n):
        a, b = (u - 1) % n, (u + 1) % n
        ci += [min(a, b), max(a, b)]
        ro.append(len(ci))
    return ro, ci


def star_csr(n: int):
    """star_graph (generators.rs:421-449)."""
    ro, ci = [0], list(range(1, n))
    ro.append(len(ci))
    for _ in range(1, n):
        ci.append(0)
        ro.append(len(ci))
    return ro, ci


def cliques_csr(sizes):
    """disconnected_cliques (generators.rs:513-544)."""
    ro, ci, base = [0], [], 0
    for k in sizes:
        for u in range(k):
            ci += [base + v for v in range(k) if v != u]
            ro.append(len(ci))
        base += k
    return ro, ci


def case(name, ref, V, ro, ci, sources, dist, **extra):
    d = {"name": name, "reference": ref, "num_vertices": V, "row_offsets": ro,
         "col_indices": ci, "sources": list(sources), "dist": dist}
    d.update(extra)
    return d


def main() -> None:
    cases = []

    # --- BFS known answers -------------------------------------------------
    for (w, h, srcs, ref) in [
        (3, 3, [0, 4, 8], "crates/core/src/generators.rs:646-663 (3x3 sources 0,4,8)"),
        (10, 10, [0, 99, 45], "crates/core/src/generators.rs:631-644 (10x10, d(0,99)=18)"),
        (6, 6, [(i * 2) % 36 for i in range(17)],
         "tests/tier2_boundaries/b6_batch_sizes.rs:14-22 (6x6 grid, S=17)"),
        (4, 3, [0, 5, 11], "crates/core/src/generators.rs:595-608 (4x3 grid)"),
        (16, 16, [(i * 61 + 7) % 256 for i in range(64)],
         "Grid2D Manhattan oracle (generators.rs:95-127), S=64: two 32-lane words"),
    ]:
        ro, ci = grid_csr(w, h)
        V = w * h
        cases.append(case(f"grid_{w}x{h}_s{len(srcs)}", ref, V, ro, ci, srcs,
                          manhattan(w, srcs, V), symmetric=True))

    # Directed cycle i -> i+1 (mod N): d(s, v) = (v - s) mod N.
    N = 100
    ro, ci = edges_to_csr(N, [(i, (i + 1) % N) for i in range(N)])
    for S in (1, 32, 64, 100):
        srcs = [(i * 7) % N for i in range(S)]
        dist = [(v + N - s) % N for s in srcs for v in range(N)]
        cases.append(case(f"directed_cycle_100_s{S}",
                          "crates/gpu_bfs/tests/m9_adversarial_stress.rs:407-430",
                          N, ro, ci, srcs, dist, symmetric=False))

    # Path graphs: d(0, v) = v (tier2 b7_01 / b7_02); both ends (b7_03).
    for n, srcs, ref in [(50, [0], "tests/tier2_boundaries/b7_extreme_diameters.rs:6-16"),
                         (120, [0], "tests/tier2_boundaries/b7_extreme_diameters.rs:18-28"),
                         (60, [0, 59], "tests/tier2_boundaries/b7_extreme_diameters.rs:30-37")]:
        ro, ci = path_csr(n)
        cases.append(case(f"path_{n}_s{len(srcs)}", ref, n, ro, ci, srcs,
                          [abs(v - s) for s in srcs for v in range(n)], symmetric=True))

    # Undirected cycle of 60 from 0: min(v, 60 - v) (b7_04).
    ro, ci = cycle_csr(60)
    cases.append(case("cycle_60_s1", "tests/tier2_boundaries/b7_extreme_diameters.rs:39-50",
                      60, ro, ci, [0], [min(v, 60 - v) for v in range(60)], symmetric=True))

    # Star: hub 0 at distance 1 from every leaf, leaves 2 apart.
    n = 200
    ro, ci = star_csr(n)
    srcs = [0, 1, 150]
    dist = []
    for s in srcs:
        dist += [0 if v == s else (1 if (s == 0 or v == 0) else 2) for v in range(n)]
    cases.append(case("star_200_s3", "crates/core/src/generators.rs:421-449 (hub contention)",
                      n, ro, ci, srcs, dist, symmetric=True))

    # Disconnected cliques: 1 inside a clique, unreachable across.
    sizes = [5, 7, 3]
    ro, ci = cliques_csr(sizes)
    V = sum(sizes)
    comp = [i for i, k in enumerate(sizes) for _ in range(k)]
    srcs = [0, 6, 14, 2]
    dist = [0 if v == s else (1 if comp[v] == comp[s] else MAX) for s in srcs for v in range(V)]
    cases.append(case("disconnected_cliques_5_7_3", "tests/tier2_boundaries/"
                      "b5_disconnected_components.rs", V, ro, ci, srcs, dist, symmetric=True))

    # Isolated vertices (zero edges): only the source itself is reachable.
    V = 9
    srcs = [0, 4, 4, 8]
    dist = [0 if v == s else MAX for s in srcs for v in range(V)]
    cases.append(case("isolated_9_duplicate_sources", "tests/tier2_boundaries/b3_zero_edges.rs",
                      V, [0] * (V + 1), [], srcs, dist, symmetric=True))

    # Feed-forward DAG u -> v (u < v, (u + v) % 5 == 0): source 49 (out-degree 0)
    # reaches only itself (tests/tier3_combinations/t3_03_asymmetric_pushpull.rs:23-52).
    V = 50
    edges = [(u, v) for u in range(V) for v in range(u + 1, V) if (u + v) % 5 == 0]
    ro, ci = edges_to_csr(V, edges)
    cases.append(case("dag_50_source_49", "tests/tier3_combinations/"
                      "t3_03_asymmetric_pushpull.rs:23-52", V, ro, ci, [49],
                      [MAX] * 49 + [0], symmetric=False))

    # --- graph-core literals ------------------------------------------------
    core = {
        "csr_construction": {
            "reference": "crates/core/src/graph.rs:653-673",
            "num_vertices": 3, "edges": [[0, 1], [0, 2], [1, 2], [2, 0]],
            "row_offsets": [0, 2, 3, 4], "col_indices": [1, 2, 2, 0], "max_degree": 2},
        "self_loops_and_duplicates": {
            "reference": "crates/core/src/graph.rs:675-692",
            "num_vertices": 3, "edges": [[0, 0], [0, 1], [0, 1], [1, 2], [2, 2]],
            "row_offsets": [0, 1, 2, 2], "col_indices": [1, 2]},
        "transpose": {
            "reference": "crates/core/src/graph.rs:694-715",
            "num_vertices": 3, "edges": [[0, 1], [0, 2], [1, 2]],
            "col_offsets": [0, 0, 1, 3], "row_indices": [0, 0, 1]},
        "symmetry": {
            "reference": "crates/core/src/graph.rs:717-728",
            "asymmetric": [[0, 1], [1, 2]], "symmetric": [[0, 1], [1, 0], [1, 2], [2, 1]]},
        "to_undirected": {
            "reference": "crates/core/src/graph.rs:730-743",
            "num_vertices": 3, "edges": [[0, 1], [1, 2]],
            "row_offsets": [0, 1, 3, 4], "col_indices": [1, 0, 2, 1]},
        "reachability_bitmask": {
            "reference": "crates/core/src/graph.rs:761-797",
            "num_vertices": 5, "num_sources": 70,
            "finite": [[0, 0, 0], [33, 0, 2], [69, 4, 5]],
            "words_per_vertex": 3,
            "words": [1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 32]},
        "grid_4x3_csr": {
            "reference": "crates/core/src/generators.rs:28-80 (N, W, E, S order)",
            "width": 4, "height": 3, "row_offsets": grid_csr(4, 3)[0],
            "col_indices": grid_csr(4, 3)[1], "num_edges": 2 * (3 * 3 + 4 * 2)},
    }
    OUT.write_text(json.dumps({"bfs": cases, "core": core}, separators=(",", ":")))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(cases)} BFS cases)")


if __name__ == "__main__":
    main()
