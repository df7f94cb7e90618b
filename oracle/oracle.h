/*
 * CPU oracle for the multi-source BFS hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * CPU BFS crate (crates/cpu_bfs) and of the CSR/CSC helpers of its core crate
 * (crates/core/src/graph.rs). It is the checker for the CUDA engine: only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark may
 * load it. The engine library never links or calls it.
 *
 * Parity pinning: the restatement is checked against the reference's own
 * known-answer tests (CSR/CSC literals, Grid2D Manhattan distances, directed
 * cycle (v - s) mod N, the DAG whose out-degree-0 source reaches only itself,
 * path/star/cycle/clique/disconnected topologies and the ReachabilityBitmask
 * literals), stored as fixtures under tests/golden/. The reference's random
 * graph generators draw from rand 0.8.8 StdRng (ChaCha12) and rand_chacha
 * 0.3.1; no reference test pins generated graphs byte-for-byte, so generated
 * inputs are produced by the engine's own seeded generators and fed to both
 * sides.
 *
 * All distances are u32 hop counts, dist[s * V + v]; unreachable = 0xFFFFFFFF.
 */
#ifndef MSBFS_ORACLE_H
#define MSBFS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_OK 0
#define ORACLE_ERR_SOURCE_OOB 1
#define ORACLE_ERR_INVALID 2

/* Single-source FIFO BFS into a V-long row pre-filled with 0xFFFFFFFF.
 * Follows crates/cpu_bfs/src/fifo.rs:10-46. `queue` holds V entries. */
void oracle_bfs_single_source_into(size_t V, const uint32_t *row_offsets,
                                   const uint32_t *col_indices, uint32_t source,
                                   uint32_t *dist, uint32_t *queue);

/* Sequential multi-source FIFO BFS (fifo.rs:70-102). `out` holds S*V u32.
 * Returns ORACLE_ERR_SOURCE_OOB (index in *bad_index) if a source >= V.
 * S == 0 or V == 0 writes nothing and returns ORACLE_OK. */
int oracle_ms_bfs_fifo(size_t V, const uint32_t *row_offsets,
                       const uint32_t *col_indices, const uint32_t *sources,
                       size_t S, uint32_t *out, size_t *bad_index);

/* One FIFO BFS per source on a pool of `threads` POSIX threads, disjoint rows
 * (rayon_ms.rs:11-54). threads <= 0 means all online cores. */
int oracle_ms_bfs_threaded(size_t V, const uint32_t *row_offsets,
                           const uint32_t *col_indices, const uint32_t *sources,
                           size_t S, uint32_t *out, int threads,
                           size_t *bad_index);

/* 64-lane bit-parallel push BFS in batches of 64 sources
 * (bit_parallel.rs:11-130). */
int oracle_ms_bfs_bit_parallel(size_t V, const uint32_t *row_offsets,
                               const uint32_t *col_indices,
                               const uint32_t *sources, size_t S,
                               uint32_t *out, size_t *bad_index);

/* ReachabilityBitmask words from canonical distances (graph.rs:571-646):
 * words[v * wpv + s / 32] bit (s % 32) set iff dist[s * V + v] != MAX,
 * wpv = ceil(S / 32). `words` holds V * wpv u32. */
void oracle_reachability_from_distances(size_t V, size_t S,
                                        const uint32_t *dist, uint32_t *words);

/* Traversed edges = sum over sources of out-degrees of reached vertices
 * (crates/cli/src/bench.rs:478-491). */
uint64_t oracle_traversed_edges(size_t V, const uint32_t *row_offsets, size_t S,
                                const uint32_t *dist);

/* CsrGraph::from_edge_list (graph.rs:51-88): drop self-loops and
 * out-of-range endpoints, sort by (u, v), dedup. row_offsets holds V+1,
 * col_indices holds n_edges entries; *out_E receives the final edge count. */
void oracle_csr_from_edge_list(size_t V, size_t n_edges, const uint32_t *eu,
                               const uint32_t *ev, uint32_t *row_offsets,
                               uint32_t *col_indices, size_t *out_E);

/* CsrGraph::to_csc counting-sort transpose (graph.rs:90-127). */
void oracle_to_csc(size_t V, size_t E, const uint32_t *row_offsets,
                   const uint32_t *col_indices, uint32_t *col_offsets,
                   uint32_t *row_indices);

/* CsrGraph::is_symmetric (graph.rs:129-133): 1 when CSR == its transpose. */
int oracle_is_symmetric(size_t V, size_t E, const uint32_t *row_offsets,
                        const uint32_t *col_indices);

#ifdef __cplusplus
}
#endif

#endif
