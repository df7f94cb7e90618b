// C ABI of the host graph core and generators (include/msbfs.h, "graph core"
// and "generators" sections). Arrays handed out are malloc'd so any FFI can
// release them with msbfs_csr_free.
#include <cstdlib>
#include <cstring>
#include <new>

#include "../../include/msbfs.h"
#include "host_graph.h"

using msbfs::HostCsr;

static int export_csr(const HostCsr& g, msbfs_csr* out) {
  if (!out) return MSBFS_ERR_INVALID_ARGUMENT;
  out->num_vertices = g.V;
  out->num_edges = g.E;
  out->row_offsets = (uint32_t*)malloc((g.V + 1) * sizeof(uint32_t));
  out->col_indices = (uint32_t*)malloc((g.E ? g.E : 1) * sizeof(uint32_t));
  if (!out->row_offsets || !out->col_indices) {
    free(out->row_offsets);
    free(out->col_indices);
    out->row_offsets = out->col_indices = nullptr;
    return MSBFS_ERR_OOM;
  }
  if (g.off.empty())
    out->row_offsets[0] = 0;
  else
    memcpy(out->row_offsets, g.off.data(), (g.V + 1) * sizeof(uint32_t));
  if (g.E) memcpy(out->col_indices, g.idx.data(), g.E * sizeof(uint32_t));
  return MSBFS_OK;
}

template <typename F>
static int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return MSBFS_ERR_OOM;
  } catch (...) {
    return MSBFS_ERR_INVALID_ARGUMENT;
  }
}

extern "C" {

void msbfs_csr_free(msbfs_csr* c) {
  if (!c) return;
  free(c->row_offsets);
  free(c->col_indices);
  c->row_offsets = c->col_indices = nullptr;
  c->num_vertices = c->num_edges = 0;
}

int msbfs_csr_from_edge_list(size_t V, size_t n, const uint32_t* src, const uint32_t* dst,
                             msbfs_csr* out) {
  if (n && (!src || !dst)) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::csr_from_edge_list(V, src, dst, n), out); });
}

int msbfs_csr_transpose(const msbfs_csr* in, msbfs_csr* out) {
  if (!in || !in->row_offsets) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] {
    return export_csr(
        msbfs::transpose(in->num_vertices, in->num_edges, in->row_offsets, in->col_indices), out);
  });
}

int msbfs_csr_is_symmetric(const msbfs_csr* c) {
  if (!c || !c->row_offsets) return 0;
  return msbfs::is_symmetric(c->num_vertices, c->num_edges, c->row_offsets, c->col_indices) ? 1
                                                                                             : 0;
}

int msbfs_csr_to_undirected(const msbfs_csr* in, msbfs_csr* out) {
  if (!in || !in->row_offsets) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] {
    const size_t V = in->num_vertices;
    if (msbfs::is_symmetric(V, in->num_edges, in->row_offsets, in->col_indices)) {
      HostCsr g;
      g.V = V;
      g.E = in->num_edges;
      g.off.assign(in->row_offsets, in->row_offsets + V + 1);
      g.idx.assign(in->col_indices, in->col_indices + in->num_edges);
      return export_csr(g, out);
    }
    std::vector<uint64_t> pairs;
    pairs.reserve(in->num_edges);
    for (size_t u = 0; u < V; ++u)
      for (uint32_t e = in->row_offsets[u]; e < in->row_offsets[u + 1]; ++e)
        pairs.push_back(((uint64_t)u << 32) | in->col_indices[e]);
    return export_csr(msbfs::csr_from_pairs(V, pairs, true), out);
  });
}

int msbfs_csr_validate(const msbfs_csr* c, char* msg, size_t len) {
  if (!c) return MSBFS_ERR_INVALID_ARGUMENT;
  std::string why = msbfs::validate(c->num_vertices, c->num_edges, c->row_offsets,
                                    c->col_indices, c->num_edges);
  if (msg && len) {
    strncpy(msg, why.c_str(), len - 1);
    msg[len - 1] = 0;
  }
  return why.empty() ? MSBFS_OK : MSBFS_ERR_INVALID_GRAPH;
}

uint32_t msbfs_csr_max_degree(const msbfs_csr* c) {
  if (!c || !c->row_offsets) return 0;
  return msbfs::max_degree(c->num_vertices, c->row_offsets);
}

int msbfs_gen_grid2d(size_t w, size_t h, msbfs_csr* out) {
  if (w == 0 || h == 0) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::gen_grid2d(w, h), out); });
}

int msbfs_gen_erdos_renyi_np(size_t n, double p, uint64_t seed, msbfs_csr* out) {
  if (n == 0 || !(p >= 0.0 && p <= 1.0)) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::gen_erdos_renyi_np(n, p, seed), out); });
}

int msbfs_gen_random_tree(size_t n, uint64_t seed, msbfs_csr* out) {
  if (n == 0) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::gen_random_tree(n, seed), out); });
}

int msbfs_gen_rmat(uint32_t scale, uint32_t ef, double a, double b, double c, double d,
                   uint64_t seed, int directed, msbfs_csr* out) {
  if (scale == 0 || scale > 30) return MSBFS_ERR_INVALID_ARGUMENT;
  const double sum = a + b + c + d;
  if (sum < 1.0 - 1e-6 || sum > 1.0 + 1e-6) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded(
      [&] { return export_csr(msbfs::gen_rmat(scale, ef, a, b, c, d, seed, directed != 0), out); });
}

int msbfs_gen_path(size_t n, msbfs_csr* out) {
  return guarded([&] { return export_csr(msbfs::gen_path(n), out); });
}
int msbfs_gen_star(size_t n, msbfs_csr* out) {
  return guarded([&] { return export_csr(msbfs::gen_star(n), out); });
}
int msbfs_gen_cycle(size_t n, msbfs_csr* out) {
  return guarded([&] { return export_csr(msbfs::gen_cycle(n), out); });
}
int msbfs_gen_clique(size_t n, msbfs_csr* out) {
  return guarded([&] { return export_csr(msbfs::gen_clique(n), out); });
}
int msbfs_gen_disconnected_cliques(const size_t* sizes, size_t count, msbfs_csr* out) {
  if (count && !sizes) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::gen_disconnected_cliques(sizes, count), out); });
}

int msbfs_gen_wilson_grid(size_t w, size_t h, size_t extra, uint64_t seed, msbfs_csr* out) {
  if (w == 0 || h == 0) return MSBFS_ERR_INVALID_ARGUMENT;
  return guarded([&] { return export_csr(msbfs::gen_wilson_grid(w, h, extra, seed), out); });
}

int msbfs_sample_sources(const msbfs_csr* c, size_t count, uint64_t seed, uint32_t min_degree,
                         uint32_t* out) {
  if (!c || !c->row_offsets || (count && !out)) return MSBFS_ERR_INVALID_ARGUMENT;
  return msbfs::sample_sources(c->num_vertices, c->row_offsets, count, seed, min_degree, out)
             ? MSBFS_OK
             : MSBFS_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
