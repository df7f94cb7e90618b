// Host graph core: CSR/CSC construction, validation and seeded generators.
// Restates crates/core/src/graph.rs and crates/core/src/generators.rs of the
// reference in C++17; the big builders (R-MAT symmetrisation, transpose) run
// on all host cores because the benchmark graphs (R-MAT scale 22-24, up to
// half a billion directed edges) are built before every benchmark.
#include "host_graph.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <cstdlib>
#include <thread>

namespace msbfs {

int host_threads() {
  unsigned n = std::thread::hardware_concurrency();
  // MSBFS_HOST_THREADS caps the host-side parallel work (graph building,
  // the Matrix Market reader) for processes that share the host's cores.
  if (const char* e = getenv("MSBFS_HOST_THREADS")) {
    const int v = atoi(e);
    if (v > 0) n = (unsigned)v;
  }
  if (n == 0) n = 1;
  if (n > 64) n = 64;
  return (int)n;
}

// Runs body(t, begin, end) over [0, n) split into contiguous chunks.
static void parallel_for(size_t n, const std::function<void(int, size_t, size_t)>& body,
                         size_t min_chunk = 1 << 16) {
  int nt = host_threads();
  if (n < min_chunk * 2 || nt == 1) {
    body(0, 0, n);
    return;
  }
  size_t max_t = (n + min_chunk - 1) / min_chunk;
  if ((size_t)nt > max_t) nt = (int)max_t;
  std::vector<std::thread> th;
  size_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    size_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back(body, t, b, e);
  }
  for (auto& x : th) x.join();
}

// Dynamic schedule over [0, n) in blocks of `grain` (per-vertex work is skewed
// on power-law graphs).
static void parallel_dynamic(size_t n, size_t grain,
                             const std::function<void(size_t, size_t)>& body) {
  int nt = host_threads();
  if (n <= grain || nt == 1) {
    body(0, n);
    return;
  }
  std::atomic<size_t> cursor{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&] {
      for (;;) {
        size_t b = cursor.fetch_add(grain);
        if (b >= n) break;
        body(b, std::min(n, b + grain));
      }
    });
  for (auto& x : th) x.join();
}

HostCsr csr_from_edge_list(size_t V, const uint32_t* u, const uint32_t* v, size_t n) {
  std::vector<uint64_t> pairs;
  pairs.reserve(n);
  for (size_t i = 0; i < n; ++i) pairs.push_back(((uint64_t)u[i] << 32) | v[i]);
  return csr_from_pairs(V, pairs, false);
}

HostCsr csr_from_pairs(size_t V, const std::vector<uint64_t>& pairs, bool symmetrise) {
  HostCsr g;
  g.V = V;
  g.off.assign(V + 1, 0);
  if (V == 0) return g;
  const size_t n = pairs.size();
  // 1. degree count (both directions when symmetrising)
  std::vector<std::atomic<uint32_t>> deg(V);
  for (size_t i = 0; i < V; ++i) deg[i].store(0, std::memory_order_relaxed);
  parallel_for(n, [&](int, size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      uint32_t a = (uint32_t)(pairs[i] >> 32), c = (uint32_t)pairs[i];
      if (a == c || a >= V || c >= V) continue;
      deg[a].fetch_add(1, std::memory_order_relaxed);
      if (symmetrise) deg[c].fetch_add(1, std::memory_order_relaxed);
    }
  });
  std::vector<uint64_t> raw_off(V + 1, 0);
  for (size_t i = 0; i < V; ++i) raw_off[i + 1] = raw_off[i] + deg[i].load(std::memory_order_relaxed);
  const uint64_t raw_E = raw_off[V];
  // 2. scatter
  std::vector<uint32_t> raw(raw_E ? raw_E : 1);
  for (size_t i = 0; i < V; ++i) deg[i].store(0, std::memory_order_relaxed);
  parallel_for(n, [&](int, size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      uint32_t a = (uint32_t)(pairs[i] >> 32), c = (uint32_t)pairs[i];
      if (a == c || a >= V || c >= V) continue;
      raw[raw_off[a] + deg[a].fetch_add(1, std::memory_order_relaxed)] = c;
      if (symmetrise) raw[raw_off[c] + deg[c].fetch_add(1, std::memory_order_relaxed)] = a;
    }
  });
  // 3. per-vertex sort + dedup (generators.rs:575-580)
  std::vector<uint32_t> cnt(V, 0);
  parallel_dynamic(V, 4096, [&](size_t b, size_t e) {
    for (size_t x = b; x < e; ++x) {
      uint32_t* lo = raw.data() + raw_off[x];
      uint32_t* hi = raw.data() + raw_off[x + 1];
      std::sort(lo, hi);
      cnt[x] = (uint32_t)(std::unique(lo, hi) - lo);
    }
  });
  // 4. compact
  for (size_t i = 0; i < V; ++i) g.off[i + 1] = g.off[i] + cnt[i];
  g.E = g.off[V];
  g.idx.resize(g.E);
  parallel_dynamic(V, 4096, [&](size_t b, size_t e) {
    for (size_t x = b; x < e; ++x)
      if (cnt[x])
        std::memcpy(g.idx.data() + g.off[x], raw.data() + raw_off[x], cnt[x] * sizeof(uint32_t));
  });
  return g;
}

HostCsr csr_from_pair_lists(size_t V, const std::vector<const std::vector<uint64_t>*>& lists) {
  HostCsr g;
  g.V = V;
  g.off.assign(V + 1, 0);
  if (V == 0) return g;
  const int T = host_threads();
  // Slices of the input lists, the unit of the two parallel passes below.
  struct Slice {
    const uint64_t* p;
    size_t n;
  };
  size_t n = 0;
  for (const auto* l : lists) n += l->size();
  const size_t piece = std::max<size_t>(size_t(1) << 16, (n + 4 * (size_t)T - 1) / (4 * (size_t)T));
  std::vector<Slice> slices;
  for (const auto* l : lists)
    for (size_t b = 0; b < l->size(); b += piece)
      slices.push_back(Slice{l->data() + b, std::min(piece, l->size() - b)});
  // Partitions: P = 2^pbits contiguous source ranges of 2^shift vertices.
  unsigned bits = 0;
  while ((size_t(1) << bits) < V) ++bits;
  unsigned pbits = 0;
  while ((size_t(1) << pbits) < 8 * (size_t)T && pbits < bits) ++pbits;
  const unsigned shift = bits - pbits;
  const size_t P = size_t(1) << pbits;
  const size_t S = slices.size();
  auto valid = [V](uint64_t x) {
    const uint32_t a = (uint32_t)(x >> 32), c = (uint32_t)x;
    return a != c && a < V && c < V;
  };
  // 1. per-slice histogram of partitions
  std::vector<uint64_t> hist(S * P, 0);
  parallel_dynamic(S, 1, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      uint64_t* h = hist.data() + i * P;
      for (size_t k = 0; k < slices[i].n; ++k) {
        const uint64_t x = slices[i].p[k];
        if (valid(x)) ++h[(x >> 32) >> shift];
      }
    }
  });
  // 2. write cursors, partition-major then slice: each partition's pairs
  // end up contiguous in `part`
  std::vector<uint64_t> pbase(P + 1, 0);
  uint64_t m = 0;
  for (size_t q = 0; q < P; ++q) {
    pbase[q] = m;
    for (size_t i = 0; i < S; ++i) {
      const uint64_t c = hist[i * P + q];
      hist[i * P + q] = m;
      m += c;
    }
  }
  pbase[P] = m;
  std::vector<uint64_t> part(m ? m : 1);
  parallel_dynamic(S, 1, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      uint64_t* h = hist.data() + i * P;
      for (size_t k = 0; k < slices[i].n; ++k) {
        const uint64_t x = slices[i].p[k];
        if (valid(x)) part[h[(x >> 32) >> shift]++] = x;
      }
    }
  });
  // 3. each partition: degrees, offsets and targets of its own vertices
  std::vector<uint32_t> raw(m ? m : 1);
  std::vector<uint64_t> raw_off(V + 1, 0);
  raw_off[V] = m;
  parallel_dynamic(P, 1, [&](size_t b, size_t e) {
    std::vector<uint32_t> cur;
    for (size_t q = b; q < e; ++q) {
      const size_t lo = q << shift, hi = std::min(V, (q + 1) << shift);
      if (lo >= hi) continue;
      cur.assign(hi - lo, 0);
      for (uint64_t k = pbase[q]; k < pbase[q + 1]; ++k) ++cur[(part[k] >> 32) - lo];
      uint64_t run = pbase[q];
      for (size_t u = lo; u < hi; ++u) {
        raw_off[u] = run;
        run += cur[u - lo];
        cur[u - lo] = 0;
      }
      for (uint64_t k = pbase[q]; k < pbase[q + 1]; ++k) {
        const size_t u = (size_t)(part[k] >> 32);
        raw[raw_off[u] + cur[u - lo]++] = (uint32_t)part[k];
      }
    }
  });
  std::vector<uint64_t>().swap(part);
  // 4. per-vertex sort + dedup, 5. compact (as csr_from_pairs)
  std::vector<uint32_t> cnt(V, 0);
  parallel_dynamic(V, 4096, [&](size_t b, size_t e) {
    for (size_t x = b; x < e; ++x) {
      uint32_t* lo = raw.data() + raw_off[x];
      uint32_t* hi = raw.data() + raw_off[x + 1];
      std::sort(lo, hi);
      cnt[x] = (uint32_t)(std::unique(lo, hi) - lo);
    }
  });
  for (size_t i = 0; i < V; ++i) g.off[i + 1] = g.off[i] + cnt[i];
  g.E = g.off[V];
  g.idx.resize(g.E);
  parallel_dynamic(V, 4096, [&](size_t b, size_t e) {
    for (size_t x = b; x < e; ++x)
      if (cnt[x])
        std::memcpy(g.idx.data() + g.off[x], raw.data() + raw_off[x], cnt[x] * sizeof(uint32_t));
  });
  return g;
}

HostCsr transpose(size_t V, size_t E, const uint32_t* off, const uint32_t* idx) {
  HostCsr t;
  t.V = V;
  t.E = E;
  t.off.assign(V + 1, 0);
  t.idx.resize(E);
  for (size_t e = 0; e < E; ++e) t.off[idx[e] + 1]++;
  for (size_t i = 0; i < V; ++i) t.off[i + 1] += t.off[i];
  std::vector<uint32_t> pos(t.off.begin(), t.off.end() - (V ? 1 : 0));
  for (size_t u = 0; u < V; ++u)
    for (uint32_t e = off[u]; e < off[u + 1]; ++e) t.idx[pos[idx[e]]++] = (uint32_t)u;
  return t;
}

bool is_symmetric(size_t V, size_t E, const uint32_t* off, const uint32_t* idx) {
  HostCsr t = transpose(V, E, off, idx);
  return std::equal(t.off.begin(), t.off.end(), off) &&
         (E == 0 || std::memcmp(t.idx.data(), idx, E * sizeof(uint32_t)) == 0);
}

std::string validate(size_t V, size_t E, const uint32_t* off, const uint32_t* idx,
                     size_t idx_len) {
  char buf[256];
  if (!off) return "row_offsets is null";
  if (off[0] != 0) {
    snprintf(buf, sizeof buf, "row_offsets[0] must be 0, got %u", off[0]);
    return buf;
  }
  for (size_t i = 0; i < V; ++i)
    if (off[i] > off[i + 1]) {
      snprintf(buf, sizeof buf, "row_offsets not monotonic at %zu: %u > %u", i, off[i],
               off[i + 1]);
      return buf;
    }
  if ((size_t)off[V] != idx_len || (size_t)off[V] != E) {
    snprintf(buf, sizeof buf, "edge count mismatch: last offset %u, col_indices length %zu",
             off[V], idx_len);
    return buf;
  }
  if (E && !idx) return "col_indices is null";
  for (size_t e = 0; e < E; ++e)
    if (idx[e] >= V) {
      snprintf(buf, sizeof buf, "col_indices[%zu] = %u out of bounds for %zu vertices", e,
               idx[e], V);
      return buf;
    }
  for (size_t u = 0; u < V; ++u)
    for (uint32_t e = off[u] + 1; e < off[u + 1]; ++e)
      if (idx[e - 1] >= idx[e]) {
        snprintf(buf, sizeof buf,
                 "unsorted or duplicate neighbours of vertex %zu: %u then %u", u,
                 idx[e - 1], idx[e]);
        return buf;
      }
  return std::string();
}

std::string graph_class(size_t V, size_t E, uint32_t max_deg) {
  const char* kind = (max_deg <= 8 && E <= 4 * V) ? "road" : (max_deg >= 128 ? "powerlaw" : "mesh");
  int lv = 0;
  while ((size_t(1) << (lv + 1)) <= V) ++lv;
  return std::string(kind) + "/v2^" + std::to_string(lv / 2 * 2);
}

uint32_t max_degree(size_t V, const uint32_t* off) {
  uint32_t m = 0;
  for (size_t u = 0; u < V; ++u) m = std::max(m, off[u + 1] - off[u]);
  return m;
}

// ---------------------------------------------------------------- generators

HostCsr gen_grid2d(size_t w, size_t h) {
  HostCsr g;
  g.V = w * h;
  g.off.reserve(g.V + 1);
  g.off.push_back(0);
  for (size_t y = 0; y < h; ++y)
    for (size_t x = 0; x < w; ++x) {
      size_t v = y * w + x;
      if (y > 0) g.idx.push_back((uint32_t)(v - w));      // North
      if (x > 0) g.idx.push_back((uint32_t)(v - 1));      // West
      if (x + 1 < w) g.idx.push_back((uint32_t)(v + 1));  // East
      if (y + 1 < h) g.idx.push_back((uint32_t)(v + w));  // South
      g.off.push_back((uint32_t)g.idx.size());
    }
  g.E = g.idx.size();
  return g;
}

static HostCsr isolated(size_t n) {
  HostCsr g;
  g.V = n;
  g.off.assign(n + 1, 0);
  return g;
}

HostCsr gen_erdos_renyi_np(size_t n, double p, uint64_t seed) {
  if (n <= 1 || p <= 0.0) return isolated(n);
  SplitMix64 rng(seed);
  std::vector<uint64_t> pairs;
  if (p >= 0.5) {
    for (size_t u = 0; u + 1 < n; ++u)
      for (size_t v = u + 1; v < n; ++v)
        if (rng.uniform() < p) pairs.push_back(((uint64_t)u << 32) | v);
  } else {
    // Batagelj-Brandes geometric skipping over the pairs (w < v) in row-major
    // order. The reference's variant (generators.rs:163-187) moves to row u+1
    // at column v - (n-1-u) + (u+1), which skips u candidates per row and
    // realises about half of p(n-1); this one keeps every pair at probability p.
    const double log_q = std::log(1.0 - p);
    int64_t v = 1, w = -1;
    const int64_t N = (int64_t)n;
    while (v < N) {
      double r = 1.0 - rng.uniform();  // (0, 1]
      w += 1 + (int64_t)std::floor(std::log(r) / log_q);
      while (w >= v && v < N) {
        w -= v;
        v += 1;
      }
      if (v < N) pairs.push_back(((uint64_t)v << 32) | (uint64_t)w);
    }
  }
  return csr_from_pairs(n, pairs, true);
}

HostCsr gen_random_tree(size_t n, uint64_t seed) {
  if (n <= 1) return isolated(n);
  SplitMix64 rng(seed);
  std::vector<uint32_t> perm(n);
  for (size_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
  for (size_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[rng.below(i + 1)]);
  std::vector<uint64_t> pairs;
  pairs.reserve(n - 1);
  for (size_t i = 1; i < n; ++i)
    pairs.push_back(((uint64_t)perm[i] << 32) | perm[rng.below(i)]);
  return csr_from_pairs(n, pairs, true);
}

HostCsr gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                 double d, uint64_t seed, bool directed) {
  (void)d;
  const size_t V = (size_t)1 << scale;
  const size_t M = (size_t)edge_factor * V;
  const double ta = a, tb = a + b, tc = a + b + c;
  std::vector<uint64_t> pairs(M);
  // Edge i draws from its own splitmix stream, so the graph does not depend on
  // the number of threads.
  parallel_for(M, [&](int, size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; ++i) {
      SplitMix64 rng(seed * 0x9E3779B97F4A7C15ull + i * 0xD1B54A32D192ED03ull + 1);
      uint32_t u = 0, v = 0;
      for (int step = (int)scale - 1; step >= 0; --step) {
        const uint32_t bit = 1u << step;
        const double r = rng.uniform();
        if (r < ta) {
        } else if (r < tb) {
          v |= bit;
        } else if (r < tc) {
          u |= bit;
        } else {
          u |= bit;
          v |= bit;
        }
      }
      pairs[i] = ((uint64_t)u << 32) | v;  // self-loops dropped by csr_from_pairs
    }
  });
  return csr_from_pairs(V, pairs, !directed);
}

HostCsr gen_path(size_t n) {
  if (n <= 1) return isolated(n);
  HostCsr g;
  g.V = n;
  g.off.push_back(0);
  for (size_t u = 0; u < n; ++u) {
    if (u > 0) g.idx.push_back((uint32_t)(u - 1));
    if (u + 1 < n) g.idx.push_back((uint32_t)(u + 1));
    g.off.push_back((uint32_t)g.idx.size());
  }
  g.E = g.idx.size();
  return g;
}

HostCsr gen_star(size_t n) {
  if (n <= 1) return isolated(n);
  HostCsr g;
  g.V = n;
  g.off.push_back(0);
  for (size_t leaf = 1; leaf < n; ++leaf) g.idx.push_back((uint32_t)leaf);
  g.off.push_back((uint32_t)g.idx.size());
  for (size_t leaf = 1; leaf < n; ++leaf) {
    g.idx.push_back(0);
    g.off.push_back((uint32_t)g.idx.size());
  }
  g.E = g.idx.size();
  return g;
}

HostCsr gen_cycle(size_t n) {
  if (n <= 2) return gen_path(n);
  HostCsr g;
  g.V = n;
  g.off.push_back(0);
  for (size_t u = 0; u < n; ++u) {
    size_t prev = u == 0 ? n - 1 : u - 1, next = u + 1 == n ? 0 : u + 1;
    g.idx.push_back((uint32_t)std::min(prev, next));
    g.idx.push_back((uint32_t)std::max(prev, next));
    g.off.push_back((uint32_t)g.idx.size());
  }
  g.E = g.idx.size();
  return g;
}

HostCsr gen_clique(size_t n) {
  if (n <= 1) return isolated(n);
  size_t sz[1] = {n};
  return gen_disconnected_cliques(sz, 1);
}

HostCsr gen_disconnected_cliques(const size_t* sizes, size_t count) {
  HostCsr g;
  size_t total = 0;
  for (size_t i = 0; i < count; ++i) total += sizes[i];
  g.V = total;
  g.off.push_back(0);
  size_t base = 0;
  for (size_t i = 0; i < count; ++i) {
    for (size_t u = 0; u < sizes[i]; ++u) {
      for (size_t v = 0; v < sizes[i]; ++v)
        if (u != v) g.idx.push_back((uint32_t)(base + v));
      g.off.push_back((uint32_t)g.idx.size());
    }
    base += sizes[i];
  }
  g.E = g.idx.size();
  return g;
}

HostCsr gen_wilson_grid(size_t w, size_t h, size_t extra_edges, uint64_t seed) {
  const size_t n = w * h;
  if (n <= 1) return isolated(n);
  SplitMix64 rng(seed);
  // Wilson's algorithm: loop-erased random walks into the growing tree.
  std::vector<uint8_t> in_tree(n, 0);
  std::vector<uint32_t> next(n, 0);
  in_tree[rng.below(n)] = 1;
  auto step = [&](uint32_t v) -> uint32_t {
    size_t x = v % w, y = v / w;
    uint32_t nb[4];
    int k = 0;
    if (y > 0) nb[k++] = (uint32_t)(v - w);
    if (x > 0) nb[k++] = v - 1;
    if (x + 1 < w) nb[k++] = v + 1;
    if (y + 1 < h) nb[k++] = (uint32_t)(v + w);
    return nb[rng.below((uint64_t)k)];
  };
  std::vector<uint64_t> pairs;
  pairs.reserve(n - 1 + extra_edges);
  // Tree edges are stored as (min, max) keys so non-tree grid edges can be
  // enumerated below.
  std::vector<uint64_t> tree_keys;
  tree_keys.reserve(n - 1);
  for (size_t i = 0; i < n; ++i) {
    uint32_t u = (uint32_t)i;
    while (!in_tree[u]) {
      next[u] = step(u);
      u = next[u];
    }
    u = (uint32_t)i;
    while (!in_tree[u]) {
      in_tree[u] = 1;
      uint32_t a = std::min(u, next[u]), b = std::max(u, next[u]);
      tree_keys.push_back(((uint64_t)a << 32) | b);
      u = next[u];
    }
  }
  std::sort(tree_keys.begin(), tree_keys.end());
  // Enumerate grid edges (right and down) not in the tree; draw extras
  // uniformly without replacement (partial Fisher-Yates).
  std::vector<uint64_t> spare;
  spare.reserve(2 * n);
  for (size_t y = 0; y < h; ++y)
    for (size_t x = 0; x < w; ++x) {
      uint32_t v = (uint32_t)(y * w + x);
      if (x + 1 < w) {
        uint64_t key = ((uint64_t)v << 32) | (v + 1);
        if (!std::binary_search(tree_keys.begin(), tree_keys.end(), key)) spare.push_back(key);
      }
      if (y + 1 < h) {
        uint64_t key = ((uint64_t)v << 32) | (uint32_t)(v + w);
        if (!std::binary_search(tree_keys.begin(), tree_keys.end(), key)) spare.push_back(key);
      }
    }
  size_t take = std::min(extra_edges, spare.size());
  for (size_t i = 0; i < take; ++i) std::swap(spare[i], spare[i + rng.below(spare.size() - i)]);
  pairs = tree_keys;
  pairs.insert(pairs.end(), spare.begin(), spare.begin() + take);
  return csr_from_pairs(n, pairs, true);
}

bool sample_sources(size_t V, const uint32_t* off, size_t count, uint64_t seed,
                    uint32_t min_degree, uint32_t* out) {
  std::vector<uint32_t> cand;
  cand.reserve(V);
  for (size_t v = 0; v < V; ++v)
    if (off[v + 1] - off[v] >= min_degree) cand.push_back((uint32_t)v);
  if (count > cand.size()) return false;
  SplitMix64 rng(seed ^ 0x5DEECE66Dull);
  for (size_t i = 0; i < count; ++i) std::swap(cand[i], cand[i + rng.below(cand.size() - i)]);
  std::sort(cand.begin(), cand.begin() + count);
  std::memcpy(out, cand.data(), count * sizeof(uint32_t));
  return true;
}

}  // namespace msbfs
