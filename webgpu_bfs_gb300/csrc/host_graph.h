// Host-side graph core shared by the engine and the C ABI wrappers.
// Mirrors crates/core/src/graph.rs (CsrGraph / CscGraph) and
// crates/core/src/generators.rs of the reference, restated in C++17.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace msbfs {

struct HostCsr {
  size_t V = 0;
  size_t E = 0;
  std::vector<uint32_t> off;  // V + 1
  std::vector<uint32_t> idx;  // E
};

// Deterministic counter-based generator: splitmix64 over (seed, stream).
struct SplitMix64 {
  uint64_t state;
  explicit SplitMix64(uint64_t seed) : state(seed) {}
  uint64_t next() {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // Uniform double in [0, 1) with 53 random bits.
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // Uniform integer in [0, n) (Lemire's multiply-shift, bias < 2^-32 for n < 2^32).
  uint64_t below(uint64_t n) {
    return (uint64_t)(((unsigned __int128)next() * n) >> 64);
  }
};

// Number of worker threads for host-side builders.
int host_threads();

// CsrGraph::from_edge_list (graph.rs:51-79): filter, sort, dedup.
HostCsr csr_from_edge_list(size_t V, const uint32_t* u, const uint32_t* v, size_t n);
// csr_from_directed_pairs / csr_from_undirected_pairs (generators.rs:547-588),
// parallel: per-vertex adjacency sort + dedup. `pairs` holds (u, v) packed as
// u << 32 | v. Self-loops and out-of-range endpoints are dropped.
HostCsr csr_from_pairs(size_t V, const std::vector<uint64_t>& pairs, bool symmetrise);
// The same CSR from several lists of (u << 32 | v) pairs taken as one edge
// list, without concatenating them and without atomics: the pairs are
// radix-partitioned by source vertex range, then each range is built by one
// thread. Needs 8 bytes of scratch per pair.
HostCsr csr_from_pair_lists(size_t V, const std::vector<const std::vector<uint64_t>*>& lists);
// CsrGraph::to_csc (graph.rs:90-127), counting-sort transpose.
HostCsr transpose(size_t V, size_t E, const uint32_t* off, const uint32_t* idx);
// CsrGraph::is_symmetric (graph.rs:129-133).
bool is_symmetric(size_t V, size_t E, const uint32_t* off, const uint32_t* idx);
// CsrGraph::validate (graph.rs:226-280). Empty string when valid.
std::string validate(size_t V, size_t E, const uint32_t* off, const uint32_t* idx,
                     size_t idx_len);
uint32_t max_degree(size_t V, const uint32_t* off);

// Graph class of the autotuners (batched form and level path): road-like
// (max degree <= 8, E <= 4V: the router's CTA-path test), power-law (max
// degree >= 128) or mesh, and the vertex count rounded down to an even
// power of two, e.g. "powerlaw/v2^22".
std::string graph_class(size_t V, size_t E, uint32_t max_deg);

// Generators (generators.rs), seeded with SplitMix64.
HostCsr gen_grid2d(size_t w, size_t h);
HostCsr gen_erdos_renyi_np(size_t n, double p, uint64_t seed);
HostCsr gen_random_tree(size_t n, uint64_t seed);
HostCsr gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                 double d, uint64_t seed, bool directed);
HostCsr gen_path(size_t n);
HostCsr gen_star(size_t n);
HostCsr gen_cycle(size_t n);
HostCsr gen_clique(size_t n);
HostCsr gen_disconnected_cliques(const size_t* sizes, size_t count);
HostCsr gen_wilson_grid(size_t w, size_t h, size_t extra_edges, uint64_t seed);
// graph_loader.rs:132-190 random strategy, restricted to degree >= min_degree.
bool sample_sources(size_t V, const uint32_t* off, size_t count, uint64_t seed,
                    uint32_t min_degree, uint32_t* out);

}  // namespace msbfs
