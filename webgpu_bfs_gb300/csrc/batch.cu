// Batched form: many graphs of uneven size traversed in ONE persistent launch
// from a device work list, with per-graph-class configurations picked by an
// autotuner and cached.
//
// No single reference counterpart: the reference runs one graph per call
// (crates/gpu_bfs/src/engine.rs:219) and picks a method with fixed
// thresholds (select_auto_method, engine.rs:157-198; the direction switch's
// V/16 density rule, crates/shaders/src/prep_hybrid_hop.wgsl:67-71; the
// 512-source chunking, dispatch/multi_word_bp.rs:630). Here each work item is
// (graph, source range) and is run by one block:
//   ALG_BP   a block-synchronous bit-parallel BFS over up to 32*W sources:
//            per level either a top-down expansion of the frontier queue
//            (needed = f & ~vis; atomicOr; newly = needed & ~prev, as
//            indirect_sparse_push_512.wgsl:89-144) or a bottom-up scan of
//            every (vertex, word) (cand = OR of in-neighbours' frontier words
//            with early exit, as multi_word_bp_pull_512.wgsl:69-138),
//            switching on the block's own frontier count;
//   ALG_CTA  one single-source BFS per source with the visited bitmap in
//            shared memory (the workgroup-persistent design,
//            workgroup_persistent_bfs.wgsl:62-196).
// Blocks pull items from an atomic cursor; nothing waits on another block.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/msbfs.h"
#include "host_graph.h"

namespace msbfs {

enum : uint32_t { ALG_BP = 0, ALG_CTA = 1 };
enum : uint32_t { SHAPE_WORD = 0, SHAPE_VERTEX = 1 };
constexpr int BATCH_BLOCK = 512;
constexpr uint32_t BATCH_DIST_MAX = 0xffffffffu;

struct BatchGraph {
  uint32_t V, E, S;
  uint32_t alg;    // ALG_*
  uint32_t W;      // words per vertex (ALG_BP), power of two <= 8
  uint32_t div;    // ALG_BP: bottom-up when the frontier holds > V / div vertices
  uint32_t shape;  // ALG_BP tile shape: SHAPE_WORD (a thread per vertex word, a warp
                   // covers 32/W vertices x W words) or SHAPE_VERTEX (a thread per
                   // vertex with all W words, each edge list read once)
  const uint32_t* off;   // CSR
  const uint32_t* idx;
  const uint32_t* coff;  // CSC (aliases the CSR when symmetric)
  const uint32_t* cidx;
  const uint32_t* src;   // S sources
  uint32_t* dist;        // S * V
};

struct BatchItem {
  uint32_t g;   // graph
  uint32_t s0;  // first source
  uint32_t n;   // sources in this item
  uint32_t pad;
};

struct BatchParams {
  const BatchGraph* graphs;
  const BatchItem* items;
  uint32_t n_items;
  uint32_t max_levels_guard;  // unused padding for alignment
  uint32_t* cursor;
  uint32_t* scratch;          // per resident block
  size_t scratch_words;       // per block
};

__device__ __forceinline__ uint32_t bword_mask(uint32_t P, uint32_t k) {
  const uint32_t lo = k * 32;
  if (P <= lo) return 0;
  const uint32_t rem = P - lo;
  return rem >= 32 ? 0xffffffffu : ((1u << rem) - 1);
}

// Block-synchronous bit-parallel BFS of sources [s0, s0+P) of graph g.
// Scratch: vis[V*W], Fa[V*W], Fb[V*W], Qa[V], Qb[V]; sbits: V bits (shared).
template <bool VT>
__device__ void bp_item(const BatchGraph& g, uint32_t s0, uint32_t P, uint32_t* scr,
                        uint32_t* sbits, uint32_t* s_cnt) {
  const uint32_t V = g.V, W = g.W, lw = __ffs(W) - 1;
  const uint32_t VW = V * W;
  const uint32_t tid = threadIdx.x, bs = blockDim.x;
  uint32_t* vis = scr;
  uint32_t* Fa = vis + VW;
  uint32_t* Fb = Fa + VW;
  uint32_t* Qa = Fb + VW;
  uint32_t* Qb = Qa + V;
  const uint32_t bwords = (V + 31) / 32;
  for (uint32_t i = tid; i < 3 * VW; i += bs) vis[i] = 0;
  for (uint32_t i = tid; i < bwords; i += bs) sbits[i] = 0;
  if (tid == 0) {
    s_cnt[0] = 0;  // |Qa|
    s_cnt[1] = 0;  // |Qb|
  }
  __syncthreads();
  for (uint32_t i = tid; i < P; i += bs) {
    const uint32_t s = g.src[s0 + i];
    const uint32_t bit = 1u << (i & 31);
    atomicOr(&vis[(s << lw) + (i >> 5)], bit);
    atomicOr(&Fa[(s << lw) + (i >> 5)], bit);
    g.dist[(size_t)(s0 + i) * V + s] = 0;
    const uint32_t vb = 1u << (s & 31);
    if (!(atomicOr(&sbits[s >> 5], vb) & vb)) Qa[atomicAdd(&s_cnt[0], 1u)] = s;
  }
  __syncthreads();
  for (uint32_t i = tid; i < bwords; i += bs) sbits[i] = 0;
  uint32_t qa = s_cnt[0];
  __syncthreads();
  for (uint32_t L = 0; qa > 0 && L <= V; ++L) {
    const uint32_t d = L + 1;
    if (VT && (size_t)qa * g.div > V && g.shape == SHAPE_VERTEX) {
      // bottom-up, a thread per vertex: its in-edge list is read once for
      // all W words and the scan stops once every needed lane is covered.
      for (uint32_t v = tid; v < V; v += bs) {
        uint32_t needed[8], cand[8];
        uint32_t any = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
          needed[k] = k < W ? ~vis[(v << lw) + k] & bword_mask(P, k) : 0u;
          cand[k] = 0;
          any |= needed[k];
        }
        if (!any) continue;
        for (uint32_t e = g.coff[v]; e < g.coff[v + 1]; ++e) {
          const uint32_t* fu = Fa + (g.cidx[e] << lw);
          uint32_t left = 0;
#pragma unroll
          for (uint32_t k = 0; k < 8; ++k) {
            if (k < W) cand[k] |= fu[k];
            left |= needed[k] & ~cand[k];
          }
          if (!left) break;
        }
        bool found = false;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
          uint32_t newly = cand[k] & needed[k];
          if (!newly) continue;
          found = true;
          vis[(v << lw) + k] |= newly;
          Fb[(v << lw) + k] = newly;
          while (newly) {
            const uint32_t b = __ffs(newly) - 1;
            newly &= newly - 1;
            g.dist[(size_t)(s0 + k * 32 + b) * V + v] = d;
          }
        }
        if (found) {
          const uint32_t vb = 1u << (v & 31);
          if (!(atomicOr(&sbits[v >> 5], vb) & vb)) Qb[atomicAdd(&s_cnt[1], 1u)] = v;
        }
      }
    } else if ((size_t)qa * g.div > V) {
      // bottom-up: thread per (vertex, word); the owner updates its word.
      for (uint32_t i = tid; i < VW; i += bs) {
        const uint32_t v = i >> lw, k = i & (W - 1);
        const uint32_t needed = ~vis[i] & bword_mask(P, k);
        if (!needed) continue;
        uint32_t cand = 0;
        for (uint32_t e = g.coff[v]; e < g.coff[v + 1]; ++e) {
          cand |= Fa[(g.cidx[e] << lw) + k];
          if ((cand & needed) == needed) break;
        }
        uint32_t newly = cand & needed;
        if (!newly) continue;
        vis[i] |= newly;
        Fb[i] = newly;
        while (newly) {
          const uint32_t b = __ffs(newly) - 1;
          newly &= newly - 1;
          g.dist[(size_t)(s0 + k * 32 + b) * V + v] = d;
        }
        const uint32_t vb = 1u << (v & 31);
        if (!(atomicOr(&sbits[v >> 5], vb) & vb)) Qb[atomicAdd(&s_cnt[1], 1u)] = v;
      }
    } else if (VT && g.shape == SHAPE_VERTEX) {
      // top-down, a thread per frontier vertex: each out-edge's target is
      // read once for all W words.
      for (uint32_t i = tid; i < qa; i += bs) {
        const uint32_t u = Qa[i];
        uint32_t f[8];
        uint32_t any = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
          f[k] = k < W ? Fa[(u << lw) + k] : 0u;
          any |= f[k];
        }
        if (!any) continue;
        for (uint32_t e = g.off[u]; e < g.off[u + 1]; ++e) {
          const uint32_t v = g.idx[e];
          bool found = false;
#pragma unroll
          for (uint32_t k = 0; k < 8; ++k) {
            if (!f[k]) continue;
            uint32_t* vw = &vis[(v << lw) + k];
            const uint32_t needed = f[k] & ~__ldcg(vw);
            if (!needed) continue;
            uint32_t newly = needed & ~atomicOr(vw, needed);
            if (!newly) continue;
            found = true;
            atomicOr(&Fb[(v << lw) + k], newly);
            while (newly) {
              const uint32_t b = __ffs(newly) - 1;
              newly &= newly - 1;
              g.dist[(size_t)(s0 + k * 32 + b) * V + v] = d;
            }
          }
          if (found) {
            const uint32_t vb = 1u << (v & 31);
            if (!(atomicOr(&sbits[v >> 5], vb) & vb)) Qb[atomicAdd(&s_cnt[1], 1u)] = v;
          }
        }
      }
    } else {
      // top-down: thread per (frontier vertex, word).
      for (uint32_t i = tid; i < (qa << lw); i += bs) {
        const uint32_t u = Qa[i >> lw], k = i & (W - 1);
        const uint32_t f = Fa[(u << lw) + k];
        if (!f) continue;
        for (uint32_t e = g.off[u]; e < g.off[u + 1]; ++e) {
          const uint32_t v = g.idx[e];
          uint32_t* vw = &vis[(v << lw) + k];
          const uint32_t needed = f & ~__ldcg(vw);
          if (!needed) continue;
          uint32_t newly = needed & ~atomicOr(vw, needed);
          if (!newly) continue;
          atomicOr(&Fb[(v << lw) + k], newly);
          while (newly) {
            const uint32_t b = __ffs(newly) - 1;
            newly &= newly - 1;
            g.dist[(size_t)(s0 + k * 32 + b) * V + v] = d;
          }
          const uint32_t vb = 1u << (v & 31);
          if (!(atomicOr(&sbits[v >> 5], vb) & vb)) Qb[atomicAdd(&s_cnt[1], 1u)] = v;
        }
      }
    }
    __syncthreads();
    for (uint32_t i = tid; i < (qa << lw); i += bs) Fa[(Qa[i >> lw] << lw) + (i & (W - 1))] = 0;
    for (uint32_t i = tid; i < bwords; i += bs) sbits[i] = 0;
    __syncthreads();
    qa = s_cnt[1];
    uint32_t* t = Fa;
    Fa = Fb;
    Fb = t;
    t = Qa;
    Qa = Qb;
    Qb = t;
    __syncthreads();
    if (tid == 0) s_cnt[1] = 0;
    __syncthreads();
  }
  // Unreached (source, vertex) pairs, written row by row (coalesced).
  for (size_t i = tid; i < (size_t)P * V; i += bs) {
    const uint32_t s = (uint32_t)(i / V), v = (uint32_t)(i % V);
    if (!((vis[(v << lw) + (s >> 5)] >> (s & 31)) & 1u)) g.dist[(size_t)(s0 + s) * V + v] = BATCH_DIST_MAX;
  }
  __syncthreads();
}

// One single-source BFS per source of [s0, s0+n); visited bitmap in shared
// memory, frontier queues (2V) in the block's scratch.
__device__ void cta_item(const BatchGraph& g, uint32_t s0, uint32_t n, uint32_t* scr,
                         uint32_t* bitmap, uint32_t* s_cnt) {
  const uint32_t V = g.V, tid = threadIdx.x, bs = blockDim.x;
  const uint32_t bwords = (V + 31) / 32;
  for (uint32_t si = s0; si < s0 + n; ++si) {
    for (uint32_t i = tid; i < bwords; i += bs) bitmap[i] = 0;
    __syncthreads();
    const uint32_t src = g.src[si];
    uint32_t* row = g.dist + (size_t)si * V;
    uint32_t* qin = scr;
    uint32_t* qout = scr + V;
    if (tid == 0) {
      bitmap[src >> 5] = 1u << (src & 31);
      row[src] = 0;
      qin[0] = src;
      s_cnt[1] = 0;
    }
    uint32_t n_in = 1;
    __syncthreads();
    for (uint32_t L = 0; n_in; ++L) {
      for (uint32_t i = tid; i < n_in; i += bs) {
        const uint32_t u = qin[i];
        for (uint32_t e = g.off[u]; e < g.off[u + 1]; ++e) {
          const uint32_t v = g.idx[e];
          const uint32_t bit = 1u << (v & 31);
          if (bitmap[v >> 5] & bit) continue;
          if (atomicOr(&bitmap[v >> 5], bit) & bit) continue;
          row[v] = L + 1;
          qout[atomicAdd(&s_cnt[1], 1u)] = v;
        }
      }
      __syncthreads();
      n_in = s_cnt[1];
      __syncthreads();
      if (tid == 0) s_cnt[1] = 0;
      uint32_t* t = qin;
      qin = qout;
      qout = t;
      __syncthreads();
    }
    for (uint32_t v = tid; v < V; v += bs)
      if (!((bitmap[v >> 5] >> (v & 31)) & 1u)) row[v] = BATCH_DIST_MAX;
    __syncthreads();
  }
}

// VT = true compiles the vertex-tile branches in as well; their per-thread
// word arrays double the kernel's registers (and halve its occupancy), so
// a launch takes that form only when some graph's class runs vertex tiles.
template <bool VT>
__global__ void __launch_bounds__(BATCH_BLOCK) batch_kernel(BatchParams p) {
  extern __shared__ uint32_t sbits[];
  __shared__ uint32_t s_item;
  __shared__ uint32_t s_cnt[2];
  uint32_t* scr = p.scratch + (size_t)blockIdx.x * p.scratch_words;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(p.cursor, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    __syncthreads();
    if (it >= p.n_items) break;
    const BatchItem item = p.items[it];
    const BatchGraph g = p.graphs[item.g];
    if (g.alg == ALG_CTA)
      cta_item(g, item.s0, item.n, scr, sbits, s_cnt);
    else
      bp_item<VT>(g, item.s0, item.n, scr, sbits, s_cnt);
  }
}

}  // namespace msbfs

// ===================================================================== host

using namespace msbfs;

namespace {

struct ClassConfig {
  uint32_t alg = ALG_BP;
  uint32_t wcap = 8;   // ALG_BP: max words per vertex per item
  uint32_t div = 16;   // ALG_BP: bottom-up threshold
  uint32_t chunk = 4;  // ALG_CTA: sources per item
  uint32_t shape = SHAPE_WORD;  // ALG_BP: tile shape
  double ms = 0;       // tuning time of the winner
};

struct HostGraphInfo {
  size_t V, E;
  uint32_t max_deg;
  bool sym;
  std::string cls;
};

std::string class_key(size_t V, size_t E, uint32_t max_deg) {
  return msbfs::graph_class(V, E, max_deg);
}

int cuda_err(cudaError_t e) {
  if (e == cudaSuccess) return MSBFS_OK;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? MSBFS_ERR_OOM : MSBFS_ERR_CUDA;
}

#define BCK(x)                               \
  do {                                       \
    int _rc = cuda_err(x);                   \
    if (_rc) return _rc;                     \
  } while (0)

}  // namespace

struct msbfs_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<HostGraphInfo> info;
  std::vector<BatchGraph> graphs;          // device pointers filled in
  std::vector<void*> allocs;
  std::map<std::string, ClassConfig> configs;
  uint32_t* d_cursor = nullptr;
  BatchGraph* d_graphs = nullptr;
  BatchItem* d_items = nullptr;
  size_t d_items_cap = 0;
  uint32_t* d_scratch = nullptr;
  size_t scratch_words = 0;
  int grid = 0;     // resident blocks of the word-tile kernel
  int grid_vt = 0;  // and of the kernel with vertex tiles compiled in
  size_t smem = 0;
  size_t max_V = 0;
  msbfs_engine* eng = nullptr;  // plain per-graph comparison path
  std::vector<msbfs_graph*> eng_graphs;
  double last_ms = 0;
  ~msbfs_batch() {
    for (msbfs_graph* g : eng_graphs) msbfs_graph_destroy(g);
    if (eng) msbfs_engine_destroy(eng);
    for (void* a : allocs) cudaFree(a);
    if (d_items) cudaFree(d_items);
    if (d_scratch) cudaFree(d_scratch);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

// Items for graph gi under its class configuration.
void make_items(const msbfs_batch* b, uint32_t gi, const ClassConfig& c, BatchGraph& g,
                std::vector<BatchItem>& items, std::vector<double>& cost) {
  const HostGraphInfo& h = b->info[gi];
  g.alg = c.alg;
  g.div = c.div;
  g.shape = c.shape;
  if (c.alg == ALG_CTA) {
    g.W = 1;
    for (uint32_t s0 = 0; s0 < g.S; s0 += c.chunk) {
      const uint32_t n = std::min(c.chunk, g.S - s0);
      items.push_back(BatchItem{gi, s0, n, 0});
      cost.push_back((double)n * (h.V + h.E));
    }
  } else {
    uint32_t need = (g.S + 31) / 32, W = 1;
    while (W < need && W < c.wcap) W <<= 1;
    g.W = W;
    const uint32_t lanes = 32 * W;
    for (uint32_t s0 = 0; s0 < g.S; s0 += lanes) {
      const uint32_t n = std::min(lanes, g.S - s0);
      items.push_back(BatchItem{gi, s0, n, 0});
      cost.push_back((double)W * (h.V + 2.0 * h.E) * 8.0);
    }
  }
}

// Runs the listed graphs (all of them when `subset` is empty) in one launch.
int launch_batch(msbfs_batch* b, const std::vector<uint32_t>& subset, float* ms_out) {
  std::vector<BatchItem> items;
  std::vector<double> cost;
  std::vector<BatchGraph> gs = b->graphs;
  bool vt = false;
  const size_t n = subset.empty() ? b->graphs.size() : subset.size();
  for (size_t j = 0; j < n; ++j) {
    const uint32_t gi = subset.empty() ? (uint32_t)j : subset[j];
    auto it = b->configs.find(b->info[gi].cls);
    const ClassConfig c = it != b->configs.end() ? it->second : ClassConfig{};
    make_items(b, gi, c, gs[gi], items, cost);
    vt |= gs[gi].alg == ALG_BP && gs[gi].shape == SHAPE_VERTEX;
  }
  // Longest items first (LPT) so the tail of the launch is short.
  std::vector<size_t> ord(items.size());
  for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t c) { return cost[a] > cost[c]; });
  std::vector<BatchItem> sorted(items.size());
  for (size_t i = 0; i < ord.size(); ++i) sorted[i] = items[ord[i]];
  if (sorted.size() > b->d_items_cap) {
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    BCK(cudaMalloc((void**)&b->d_items, std::max<size_t>(sorted.size(), 1) * sizeof(BatchItem)));
    b->d_items_cap = sorted.size();
  }
  if (!sorted.empty())
    BCK(cudaMemcpyAsync(b->d_items, sorted.data(), sorted.size() * sizeof(BatchItem),
                        cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_graphs, gs.data(), gs.size() * sizeof(BatchGraph),
                      cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemsetAsync(b->d_cursor, 0, sizeof(uint32_t), b->stream));
  BatchParams p{};
  p.graphs = b->d_graphs;
  p.items = b->d_items;
  p.n_items = (uint32_t)sorted.size();
  p.cursor = b->d_cursor;
  p.scratch = b->d_scratch;
  p.scratch_words = b->scratch_words;
  BCK(cudaEventRecord(b->ev0, b->stream));
  const int grid = (int)std::min<size_t>((size_t)(vt ? b->grid_vt : b->grid),
                                         std::max<size_t>(sorted.size(), 1));
  if (vt)
    batch_kernel<true><<<grid, BATCH_BLOCK, b->smem, b->stream>>>(p);
  else
    batch_kernel<false><<<grid, BATCH_BLOCK, b->smem, b->stream>>>(p);
  BCK(cudaGetLastError());
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaEventSynchronize(b->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  if (ms_out) *ms_out = ms;
  return MSBFS_OK;
}

}  // namespace

extern "C" {

int msbfs_batch_create(int device, const msbfs_batch_graph* graphs, size_t n, msbfs_batch** out) {
  if (!out || (n && !graphs)) return MSBFS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd) {
    cudaGetLastError();
    return MSBFS_ERR_NO_DEVICE;
  }
  BCK(cudaSetDevice(device));
  auto b = std::make_unique<msbfs_batch>();
  b->device = device;
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreate(&b->ev0));
  BCK(cudaEventCreate(&b->ev1));
  BCK(cudaMalloc((void**)&b->d_cursor, sizeof(uint32_t)));
  b->allocs.push_back(b->d_cursor);
  size_t maxVW = 0;
  for (size_t i = 0; i < n; ++i) {
    const msbfs_batch_graph& x = graphs[i];
    if (x.num_vertices == 0 || x.num_vertices > MSBFS_BATCH_MAX_VERTICES)
      return MSBFS_ERR_INVALID_ARGUMENT;
    if (!msbfs::validate(x.num_vertices, x.num_edges, x.row_offsets, x.col_indices, x.num_edges)
             .empty())
      return MSBFS_ERR_INVALID_GRAPH;
    for (size_t s = 0; s < x.num_sources; ++s)
      if (x.sources[s] >= x.num_vertices) return MSBFS_ERR_SOURCE_OOB;
    HostGraphInfo h;
    h.V = x.num_vertices;
    h.E = x.num_edges;
    h.max_deg = msbfs::max_degree(h.V, x.row_offsets);
    msbfs::HostCsr t = msbfs::transpose(h.V, h.E, x.row_offsets, x.col_indices);
    h.sym = std::equal(t.off.begin(), t.off.end(), x.row_offsets) &&
            (h.E == 0 || std::memcmp(t.idx.data(), x.col_indices, h.E * 4) == 0);
    h.cls = class_key(h.V, h.E, h.max_deg);
    BatchGraph g{};
    g.V = (uint32_t)h.V;
    g.E = (uint32_t)h.E;
    g.S = (uint32_t)x.num_sources;
    auto up = [&](const uint32_t* src, size_t cnt, uint32_t** dst) -> int {
      BCK(cudaMalloc((void**)dst, std::max<size_t>(cnt, 1) * 4));
      b->allocs.push_back(*dst);
      if (cnt) BCK(cudaMemcpy(*dst, src, cnt * 4, cudaMemcpyHostToDevice));
      return MSBFS_OK;
    };
    uint32_t *off, *idx, *coff, *cidx, *src, *dist;
    int rc;
    if ((rc = up(x.row_offsets, h.V + 1, &off)) || (rc = up(x.col_indices, h.E, &idx))) return rc;
    if (h.sym) {
      coff = off;
      cidx = idx;
    } else if ((rc = up(t.off.data(), h.V + 1, &coff)) || (rc = up(t.idx.data(), h.E, &cidx))) {
      return rc;
    }
    if ((rc = up(x.sources, x.num_sources, &src))) return rc;
    BCK(cudaMalloc((void**)&dist, std::max<size_t>(x.num_sources * h.V, 1) * 4));
    b->allocs.push_back(dist);
    g.off = off;
    g.idx = idx;
    g.coff = coff;
    g.cidx = cidx;
    g.src = src;
    g.dist = dist;
    b->graphs.push_back(g);
    b->info.push_back(h);
    b->max_V = std::max(b->max_V, h.V);
    maxVW = std::max(maxVW, h.V);
  }
  BCK(cudaMalloc((void**)&b->d_graphs, std::max<size_t>(n, 1) * sizeof(BatchGraph)));
  b->allocs.push_back(b->d_graphs);
  // Scratch per resident block: the larger of ALG_BP (3*V*8 words + 2V) and
  // ALG_CTA (2V) for the largest graph.
  b->scratch_words = 3 * maxVW * 8 + 2 * maxVW + 64;
  b->smem = ((b->max_V + 31) / 32) * 4;
  BCK(cudaFuncSetAttribute(batch_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)std::max<size_t>(b->smem, 4)));
  BCK(cudaFuncSetAttribute(batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)std::max<size_t>(b->smem, 4)));
  int occ = 0, occ_vt = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel<false>, BATCH_BLOCK, b->smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_vt, batch_kernel<true>, BATCH_BLOCK, b->smem);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  b->grid = std::max(1, occ) * sms;
  // Scratch is per resident block; keep it within 8 GiB by running fewer
  // blocks when the largest graph is big.
  const size_t per_block = b->scratch_words * 4;
  b->grid = (int)std::max<size_t>(1, std::min<size_t>(b->grid, (size_t(8) << 30) / per_block));
  b->grid_vt = std::min(b->grid, std::max(1, occ_vt) * sms);
  BCK(cudaMalloc((void**)&b->d_scratch, (size_t)b->grid * per_block));
  *out = b.release();
  return MSBFS_OK;
}

void msbfs_batch_destroy(msbfs_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  delete b;
}

int msbfs_batch_autotune(msbfs_batch* b, size_t samples_per_class, const char* cache_path) {
  if (!b) return MSBFS_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  // Cached choices first: "class alg wcap div chunk shape ms" per line.
  std::map<std::string, ClassConfig> cached;
  if (cache_path) {
    std::ifstream in(cache_path);
    std::string cls;
    ClassConfig c;
    while (in >> cls >> c.alg >> c.wcap >> c.div >> c.chunk >> c.shape >> c.ms) cached[cls] = c;
  }
  std::map<std::string, std::vector<uint32_t>> members;
  for (uint32_t i = 0; i < b->info.size(); ++i) members[b->info[i].cls].push_back(i);
  std::vector<ClassConfig> cands;
  for (uint32_t w : {1u, 2u, 4u, 8u})
    for (uint32_t dv : {4u, 16u, 64u})
      for (uint32_t sh : {(uint32_t)SHAPE_WORD, (uint32_t)SHAPE_VERTEX}) {
        if (w == 1 && sh == SHAPE_VERTEX) continue;  // one word: the two shapes coincide
        ClassConfig c;
        c.alg = ALG_BP;
        c.wcap = w;
        c.div = dv;
        c.shape = sh;
        cands.push_back(c);
      }
  for (uint32_t ch : {1u, 4u, 16u}) {
    ClassConfig c;
    c.alg = ALG_CTA;
    c.chunk = ch;
    cands.push_back(c);
  }
  bool updated = false;
  for (auto& kv : members) {
    auto hit = cached.find(kv.first);
    if (hit != cached.end()) {
      b->configs[kv.first] = hit->second;
      continue;
    }
    // Sample: up to `samples_per_class` graphs spread over the class.
    std::vector<uint32_t> sample;
    const size_t m = kv.second.size(), k = std::max<size_t>(1, std::min(samples_per_class, m));
    for (size_t j = 0; j < k; ++j) sample.push_back(kv.second[j * m / k]);
    ClassConfig best;
    best.ms = 1e30;
    for (const ClassConfig& c : cands) {
      b->configs[kv.first] = c;
      float ms = 0;
      int rc = launch_batch(b, sample, &ms);  // warm
      if (rc) return rc;
      if ((rc = launch_batch(b, sample, &ms))) return rc;
      if (ms < best.ms) {
        best = c;
        best.ms = ms;
      }
    }
    b->configs[kv.first] = best;
    cached[kv.first] = best;
    updated = true;
  }
  if (cache_path && updated) {
    std::ofstream o(cache_path);
    for (auto& kv : cached)
      o << kv.first << " " << kv.second.alg << " " << kv.second.wcap << " " << kv.second.div
        << " " << kv.second.chunk << " " << kv.second.shape << " " << kv.second.ms << "\n";
  }
  return MSBFS_OK;
}

int msbfs_batch_run(msbfs_batch* b, double* gpu_ms) {
  if (!b) return MSBFS_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  float ms = 0;
  int rc = launch_batch(b, {}, &ms);
  if (rc) return rc;
  b->last_ms = ms;
  if (gpu_ms) *gpu_ms = ms;
  return MSBFS_OK;
}

int msbfs_batch_run_per_graph(msbfs_batch* b, const msbfs_batch_graph* graphs, double* gpu_ms) {
  if (!b || !graphs) return MSBFS_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  int rc;
  if (!b->eng) {
    if ((rc = msbfs_engine_create(b->device, MSBFS_METHOD_AUTO, &b->eng))) return rc;
    if ((rc = msbfs_engine_set_stream(b->eng, b->stream))) return rc;
    for (size_t i = 0; i < b->graphs.size(); ++i) {
      msbfs_graph* g = nullptr;
      if ((rc = msbfs_graph_create(b->eng, graphs[i].num_vertices, graphs[i].num_edges,
                                   graphs[i].row_offsets, graphs[i].col_indices, &g)))
        return rc;
      b->eng_graphs.push_back(g);
    }
  }
  BCK(cudaEventRecord(b->ev0, b->stream));
  for (size_t i = 0; i < b->graphs.size(); ++i) {
    if (graphs[i].num_sources == 0) continue;
    if ((rc = msbfs_run_ms_bfs_device(b->eng, MSBFS_METHOD_AUTO, b->eng_graphs[i],
                                      graphs[i].sources, graphs[i].num_sources,
                                      b->graphs[i].dist)))
      return rc;
  }
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaEventSynchronize(b->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  if (gpu_ms) *gpu_ms = ms;
  return MSBFS_OK;
}

int msbfs_batch_result(msbfs_batch* b, size_t i, uint32_t* out) {
  if (!b || i >= b->graphs.size() || !out) return MSBFS_ERR_INVALID_ARGUMENT;
  BCK(cudaSetDevice(b->device));
  const BatchGraph& g = b->graphs[i];
  BCK(cudaMemcpyAsync(out, g.dist, (size_t)g.S * g.V * 4, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return MSBFS_OK;
}

int msbfs_batch_config(const msbfs_batch* b, size_t i, uint32_t* alg, uint32_t* words,
                       uint32_t* param, char* class_name, size_t class_len) {
  if (!b || i >= b->info.size()) return MSBFS_ERR_INVALID_ARGUMENT;
  const std::string& cls = b->info[i].cls;
  auto it = b->configs.find(cls);
  const ClassConfig c = it != b->configs.end() ? it->second : ClassConfig{};
  if (alg) *alg = (c.alg == ALG_BP && c.shape == SHAPE_VERTEX) ? 2u : c.alg;
  if (words) *words = c.wcap;
  if (param) *param = c.alg == ALG_CTA ? c.chunk : c.div;
  if (class_name && class_len) {
    strncpy(class_name, cls.c_str(), class_len - 1);
    class_name[class_len - 1] = 0;
  }
  return MSBFS_OK;
}

}  // extern "C"
