// One-CTA-per-source persistent BFS for low-degree, high-diameter graphs
// (road networks, grids, trees).
//
// Semantics follow crates/shaders/src/workgroup_persistent_bfs.wgsl:62-196
// and crates/gpu_bfs/src/dispatch/workgroup_persistent.rs:288-370 of the
// reference: one workgroup runs a whole single-source BFS with its visited
// bitmap in shared memory and synchronises only inside the block, so a
// ~1,000-level traversal needs no grid-wide step. The GB300 form differs:
// the bitmap takes up to ~227 KB of shared memory (vs 14 KB) and, for larger
// graphs, is split over the shared memory of a thread-block cluster (calls of
// few sources) or moves to an L2-resident global slab per block instead of
// giving up the path; the frontier queues live in one L2-resident global slab of V
// words per resident block (no overflow fallback), distances are exact u32
// written into the caller's row, and the grid is persistent: each resident
// block pulls the next source from an atomic cursor until all sources are
// done. No block ever waits on another.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "../../include/msbfs.h"
#include "device_common.cuh"

namespace cg = cooperative_groups;

namespace msbfs {

constexpr uint32_t CTA_DIST_MAX = 0xffffffffu;
// Latency form's block (ms; road 339x338 + 5,000 edges S=256 / S=1, grid
// 64x64 S=64): 512 threads 1.216 / 0.964 / 0.123, 256 threads 1.148 /
// 0.912 / 0.109, 128 threads 1.402 / 1.275 / 0.109. A level of a few
// hundred frontier vertices keeps 256 threads busy, and a smaller block's
// barrier costs less.
#ifndef MSBFS_CTA_LAT_THREADS
#define MSBFS_CTA_LAT_THREADS 256
#endif
constexpr int CTA_THREADS = MSBFS_CTA_LAT_THREADS;
// Global-bitmap mode (graphs whose bitmap does not fit shared memory, e.g.
// road 1448 x 1448) keeps 512-thread blocks: its frontiers are wider.
constexpr int CTA_GB_THREADS = 512;
// Two forms. The latency form: blocks of CTA_THREADS threads, 3 resident
// per SM (4 edge records in flight, the shortest level latency). The
// throughput form, for calls with more sources than 3 blocks per SM can
// hold: CTA_TPUT_THREADS threads and CTA_TPUT_MINB resident blocks per SM
// (2 records in flight): many-source calls are bound by how many BFSs run
// at once, single ones by the per-level latency chain.
constexpr int CTA_MINB_LATENCY = 3;
// Road 339x338 + 5,000 edges, S=2048 (threads x blocks per SM, ms): 512 x 4
// 5.41, 384 x 5 4.92, 256 x 6 5.16, 256 x 7 4.46, 256 x 8 4.78, 128 x 12
// 6.68, 128 x 16 6.78. Each block waits at one barrier per level while a
// few of its warps walk a frontier of a few hundred vertices: smaller blocks
// put more sources in flight, until too few threads share a level's work.
#ifndef MSBFS_CTA_TPUT_THREADS
#define MSBFS_CTA_TPUT_THREADS 256
#endif
#ifndef MSBFS_CTA_TPUT_MINB
#define MSBFS_CTA_TPUT_MINB 7
#endif
constexpr int CTA_TPUT_THREADS = MSBFS_CTA_TPUT_THREADS;
constexpr int CTA_MINB_THROUGHPUT = MSBFS_CTA_TPUT_MINB;
static_assert(CTA_MINB_THROUGHPUT > CTA_MINB_LATENCY, "the throughput form holds more blocks");
// Global-bitmap mode keeps its per-block scratch (queue slab + bitmap) within
// this many bytes by shrinking the grid.
constexpr size_t CTA_GLOBAL_SCRATCH_BYTES = 4ull << 30;
// Frontier entries per shared-memory queue half (16 KB of vertex ids, 32 KB
// of edge ranges).
constexpr uint32_t CTA_SMEM_QUEUE = 4096;
// Cluster form: threads of rank 0 (which walks every frontier) and edge
// records each keeps in flight. Road 1448 x 1448, one source: 1,024 threads
// and 4 records 9.8 ms, 1,024 and 2 10.6 ms, 512 and 4 12.3 ms (global-bitmap
// mode 17.6 ms).
#ifndef MSBFS_CTA_CLUSTER_THREADS
#define MSBFS_CTA_CLUSTER_THREADS 1024
#endif
constexpr int CTA_CLUSTER_THREADS = MSBFS_CTA_CLUSTER_THREADS;
#ifndef MSBFS_CTA_CLUSTER_ER_BATCH
#define MSBFS_CTA_CLUSTER_ER_BATCH 4
#endif
constexpr int CTA_CLUSTER_ER_BATCH = MSBFS_CTA_CLUSTER_ER_BATCH;

// GB: the visited bitmap lives in an L2-resident global slab per block (for
// graphs whose bitmap does not fit shared memory) instead of shared memory.
//
// ER: the graph carries edge records {target, target's first edge, target's
// end edge} (built once per road-like graph), and a queue entry holds the
// edge range of a frontier vertex instead of its id. Expanding a vertex then
// costs one dependent L2 round trip per level (its edge records) instead of
// three (queue entry, offsets, adjacency): on a ~4,000-level road graph the
// per-level latency chain is what a traversal's time is made of.
//
// Queue: the first p.qh entries of a level's frontier sit in shared memory
// (two halves, by level parity), the rest in one global slab of V words per
// block (vertex ids: an ER reader looks their offsets up). The frontiers of
// consecutive levels are disjoint vertex sets, so |F_L| + |F_L+1| <= V: in
// the slab even levels sit at the front and odd levels at the back.
// Counters: level L appends through s_cnt[L % 3]; thread 0 clears
// s_cnt[(L+1) % 3] during level L (last read right after the barrier of
// level L-2), so a level needs one block barrier.
template <bool GB, bool ER, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) cta_bfs_kernel(CtaParams p) {
  constexpr int CTA_ER_BATCH = MINB >= CTA_MINB_THROUGHPUT ? 2 : 4;
  extern __shared__ __align__(16) uint32_t smem_dyn[];
  __shared__ uint32_t s_src_idx;
  __shared__ uint32_t s_cnt[3];
  __shared__ unsigned long long s_sum;
  __shared__ uint32_t s_reached;
  const uint32_t V = p.V;
  const uint32_t words = (V + 31) / 32;
  const uint32_t QH = p.qh;
  uint32_t* bits = GB ? p.gbits + (size_t)blockIdx.x * words : smem_dyn;
  // queue halves after the bitmap, 8-byte aligned: ER entries are (eb, ee)
  uint32_t* sq = smem_dyn + (GB ? 0 : (words + 1) / 2 * 2);
  uint2* sq2 = reinterpret_cast<uint2*>(sq);
  uint32_t* slab = p.gqueue + (size_t)blockIdx.x * V;
  auto slab_at = [&](uint32_t lv, uint32_t i) -> uint32_t* {
    return (lv & 1) ? slab + (V - 1 - i) : slab + i;
  };
  // Edge range [*eb, *ee) of entry i of the frontier of level `lv`.
  auto q_get = [&](uint32_t lv, uint32_t i, uint32_t* eb, uint32_t* ee) {
    if constexpr (ER) {
      if (i < QH) {
        const uint2 r = sq2[(lv & 1) * QH + i];
        *eb = r.x;
        *ee = r.y;
        return;
      }
    }
    const uint32_t u = i < QH ? sq[(lv & 1) * QH + i] : *slab_at(lv, i);
    *eb = __ldg(p.off + u);
    *ee = __ldg(p.off + u + 1);
  };
  auto q_put = [&](uint32_t lv, uint32_t i, uint32_t v, uint32_t eb, uint32_t ee) {
    if (i < QH) {
      if constexpr (ER)
        sq2[(lv & 1) * QH + i] = make_uint2(eb, ee);
      else
        sq[(lv & 1) * QH + i] = v;
    } else {
      *slab_at(lv, i) = v;
    }
  };

  for (;;) {
    if (threadIdx.x == 0) {
      s_src_idx = atomicAdd(p.work, 1u);
      s_sum = 0;
      s_reached = 0;
      s_cnt[0] = s_cnt[1] = s_cnt[2] = 0;
    }
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) bits[i] = 0;
    __syncthreads();
    const uint32_t si = s_src_idx;
    if (si >= p.num_sources) break;
    const uint32_t src = p.sources[si];
    uint32_t* row = p.dist ? p.dist + (size_t)si * V : nullptr;
    if (threadIdx.x == 0) {
      bits[src >> 5] = 1u << (src & 31);
      if (row) row[src] = 0;
      q_put(0, 0, src, __ldg(p.off + src), __ldg(p.off + src + 1));
    }
    uint32_t n_in = 1;
    uint32_t level = 0, ecc = 0;
    unsigned long long my_sum = 0;
    uint32_t my_cnt = 0;
    __syncthreads();
    while (n_in) {
      ecc = level;
      const uint32_t nd = level + 1;
      uint32_t* cnt = &s_cnt[level % 3];
      if (threadIdx.x == 0) s_cnt[(level + 1) % 3] = 0;
      // Threads sweep the frontier; each expands one vertex's out-edges.
      for (uint32_t i = threadIdx.x; i < n_in; i += blockDim.x) {
        uint32_t eb, ee;
        q_get(level, i, &eb, &ee);
        if constexpr (ER) {
          // CTA_ER_BATCH edge records in flight before any visited check
          // (road vertices have ~2 edges; more would cost registers, and so
          // resident blocks, for little gain)
          for (uint32_t e = eb; e < ee; e += CTA_ER_BATCH) {
            uint4 r[CTA_ER_BATCH];
#pragma unroll
            for (int k = 0; k < CTA_ER_BATCH; ++k)
              if (e + k < ee) r[k] = __ldg(p.erec + e + k);
#pragma unroll
            for (int k = 0; k < CTA_ER_BATCH; ++k) {
              if (e + k >= ee) break;
              const uint32_t v = r[k].x;
              const uint32_t bit = 1u << (v & 31);
              if constexpr (!GB) {
                if (bits[v >> 5] & bit) continue;
              }
              const uint32_t old = atomicOr(&bits[v >> 5], bit);
              if (old & bit) continue;
              if (row) row[v] = nd;
              my_sum += nd;
              ++my_cnt;
              q_put(level + 1, atomicAdd(cnt, 1u), v, r[k].y, r[k].z);
            }
          }
        } else {
          for (uint32_t e = eb; e < ee; ++e) {
            const uint32_t v = __ldg(p.idx + e);
            const uint32_t bit = 1u << (v & 31);
            if constexpr (!GB) {
              if (bits[v >> 5] & bit) continue;
            }
            const uint32_t old = atomicOr(&bits[v >> 5], bit);
            if (old & bit) continue;
            if (row) row[v] = nd;
            my_sum += nd;
            ++my_cnt;
            q_put(level + 1, atomicAdd(cnt, 1u), v, 0, 0);
          }
        }
      }
      __syncthreads();
      n_in = *cnt;
      ++level;
    }
    if (row) {
      // Unreached vertices: coalesced sweep of the row guided by the bitmap
      // (read from L2 in global mode: the bits were set by atomics).
      for (uint32_t v = threadIdx.x; v < V; v += blockDim.x) {
        const uint32_t w = GB ? __ldcg(bits + (v >> 5)) : bits[v >> 5];
        if (!((w >> (v & 31)) & 1u)) row[v] = CTA_DIST_MAX;
      }
    }
    if (p.stats) {
      if (my_cnt) {
        atomicAdd(&s_sum, my_sum);
        atomicAdd(&s_reached, my_cnt);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        p.stats[si].sum = s_sum;
        p.stats[si].reached = s_reached + 1;
        p.stats[si].ecc = ecc;
      }
    }
    __syncthreads();
  }
}

// Cluster form, for graphs whose visited bitmap does not fit one block's
// shared memory. A cluster of CL blocks serves one source at a time: block
// rank r keeps bitmap words [r*wpb, (r+1)*wpb) in its shared memory, and
// rank 0 runs the traversal exactly as cta_bfs_kernel does, setting visited
// bits of the other ranks' words with atomicOr through distributed shared
// memory (one hop inside the GPC instead of an L2 round trip). The other
// ranks zero their slice before a traversal and fill the unreached vertices
// of their slice after it. Two cluster barriers per source: (1) the source
// index is in every block and every slice is zero, (2) the traversal is done.
// The queue (shared-memory halves in rank 0, then one global slab of V words
// per cluster) and the edge records work as in cta_bfs_kernel.
template <int CL, bool ER>
__global__ void __launch_bounds__(CTA_CLUSTER_THREADS, 1) cta_cluster_kernel(CtaParams p) {
  constexpr int CTA_ER_BATCH = CTA_CLUSTER_ER_BATCH;
  extern __shared__ __align__(16) uint32_t smem_dyn[];
  __shared__ uint32_t s_src_idx;  // written into every block by rank 0
  __shared__ uint32_t s_cnt[3];
  __shared__ unsigned long long s_sum;
  __shared__ uint32_t s_reached;
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t rank = cluster.block_rank();
  const uint32_t V = p.V;
  const uint32_t words = (V + 31) / 32;
  const uint32_t wpb = (words + CL - 1) / CL;  // bitmap words per block
  const uint32_t w0 = min(words, rank * wpb);
  const uint32_t w1 = min(words, w0 + wpb);
  uint32_t* bits = smem_dyn;  // this block's slice: words [w0, w1)
  const uint32_t QH = p.qh;
  uint32_t* sq = smem_dyn + (wpb + 1) / 2 * 2;
  uint2* sq2 = reinterpret_cast<uint2*>(sq);
  uint32_t* slab = p.gqueue + (size_t)(blockIdx.x / CL) * V;
  auto slab_at = [&](uint32_t lv, uint32_t i) -> uint32_t* {
    return (lv & 1) ? slab + (V - 1 - i) : slab + i;
  };
  auto q_get = [&](uint32_t lv, uint32_t i, uint32_t* eb, uint32_t* ee) {
    if constexpr (ER) {
      if (i < QH) {
        const uint2 r = sq2[(lv & 1) * QH + i];
        *eb = r.x;
        *ee = r.y;
        return;
      }
    }
    const uint32_t u = i < QH ? sq[(lv & 1) * QH + i] : *slab_at(lv, i);
    *eb = __ldg(p.off + u);
    *ee = __ldg(p.off + u + 1);
  };
  auto q_put = [&](uint32_t lv, uint32_t i, uint32_t v, uint32_t eb, uint32_t ee) {
    if (i < QH) {
      if constexpr (ER)
        sq2[(lv & 1) * QH + i] = make_uint2(eb, ee);
      else
        sq[(lv & 1) * QH + i] = v;
    } else {
      *slab_at(lv, i) = v;
    }
  };
  // Word w of the whole bitmap: in this block's slice (rank 0's own) or in
  // the owning block's, reached through distributed shared memory.
  auto word_ptr = [&](uint32_t w, bool* local) -> uint32_t* {
    const uint32_t o = w / wpb;
    uint32_t* at = bits + (w - o * wpb);
    *local = o == rank;
    return *local ? at : cluster.map_shared_rank(at, o);
  };

  for (;;) {
    if (rank == 0 && threadIdx.x == 0) {
      const uint32_t si = atomicAdd(p.work, 1u);
      for (int r = 0; r < CL; ++r) *cluster.map_shared_rank(&s_src_idx, r) = si;
      s_sum = 0;
      s_reached = 0;
      s_cnt[0] = s_cnt[1] = s_cnt[2] = 0;
    }
    for (uint32_t i = threadIdx.x; i < w1 - w0; i += blockDim.x) bits[i] = 0;
    cluster.sync();  // (1)
    const uint32_t si = s_src_idx;
    if (si >= p.num_sources) break;  // the same value in every block
    const uint32_t src = p.sources[si];
    uint32_t* row = p.dist ? p.dist + (size_t)si * V : nullptr;
    uint32_t ecc = 0;
    if (rank == 0) {
      if (threadIdx.x == 0) {
        bool loc;
        atomicOr(word_ptr(src >> 5, &loc), 1u << (src & 31));
        if (row) row[src] = 0;
        q_put(0, 0, src, __ldg(p.off + src), __ldg(p.off + src + 1));
      }
      uint32_t n_in = 1;
      uint32_t level = 0;
      unsigned long long my_sum = 0;
      uint32_t my_cnt = 0;
      __syncthreads();
      while (n_in) {
        ecc = level;
        const uint32_t nd = level + 1;
        uint32_t* cnt = &s_cnt[level % 3];
        if (threadIdx.x == 0) s_cnt[(level + 1) % 3] = 0;
        for (uint32_t i = threadIdx.x; i < n_in; i += blockDim.x) {
          uint32_t eb, ee;
          q_get(level, i, &eb, &ee);
          for (uint32_t e = eb; e < ee; e += (ER ? CTA_ER_BATCH : 1)) {
            uint4 r[ER ? CTA_ER_BATCH : 1];
            if constexpr (ER) {
#pragma unroll
              for (int k = 0; k < CTA_ER_BATCH; ++k)
                if (e + k < ee) r[k] = __ldg(p.erec + e + k);
            } else {
              r[0] = make_uint4(__ldg(p.idx + e), 0u, 0u, 0u);
            }
#pragma unroll
            for (int k = 0; k < (ER ? CTA_ER_BATCH : 1); ++k) {
              if (e + k >= ee) break;
              const uint32_t v = r[k].x;
              const uint32_t bit = 1u << (v & 31);
              bool loc;
              uint32_t* wp = word_ptr(v >> 5, &loc);
              if (loc && (*wp & bit)) continue;  // a remote pre-check costs the atomic's hop
              const uint32_t old = atomicOr(wp, bit);
              if (old & bit) continue;
              if (row) row[v] = nd;
              my_sum += nd;
              ++my_cnt;
              q_put(level + 1, atomicAdd(cnt, 1u), v, r[k].y, r[k].z);
            }
          }
        }
        __syncthreads();
        n_in = *cnt;
        ++level;
      }
      if (p.stats && my_cnt) {
        atomicAdd(&s_sum, my_sum);
        atomicAdd(&s_reached, my_cnt);
      }
    }
    cluster.sync();  // (2)
    if (row) {
      // Unreached vertices of this block's slice.
      const uint32_t vb = w0 * 32, ve = min(V, w1 * 32);
      for (uint32_t v = vb + threadIdx.x; v < ve; v += blockDim.x)
        if (!((bits[(v >> 5) - w0] >> (v & 31)) & 1u)) row[v] = CTA_DIST_MAX;
    }
    if (rank == 0 && p.stats && threadIdx.x == 0) {
      p.stats[si].sum = s_sum;
      p.stats[si].reached = s_reached + 1;
      p.stats[si].ecc = ecc;
    }
    __syncthreads();  // the slice is read above and zeroed at the top
  }
}

// Edge records of a road-like graph: for every edge e = (u, v), {v, off[v],
// off[v+1], 0}. One thread per vertex u.
__global__ void edge_records_kernel(uint32_t V, const uint32_t* __restrict__ off,
                                    const uint32_t* __restrict__ idx, uint4* __restrict__ erec) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < V; u += gridDim.x * blockDim.x) {
    for (uint32_t e = off[u]; e < off[u + 1]; ++e) {
      const uint32_t v = idx[e];
      erec[e] = make_uint4(v, off[v], off[v + 1], 0u);
    }
  }
}

void launch_edge_records(uint32_t V, const uint32_t* off, const uint32_t* idx, uint4* erec,
                         cudaStream_t s) {
  edge_records_kernel<<<1024, 256, 0, s>>>(V, off, idx, erec);
}

size_t cta_max_vertices(int device) {
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  const size_t reserve = 1024;  // static shared variables and slack
  if (optin <= (int)reserve) return 0;
  return ((size_t)optin - reserve) * 8;
}

template <bool GB, bool ER, int THREADS, int MINB>
static int cta_occupancy(int block, size_t smem) {
  auto fn = cta_bfs_kernel<GB, ER, THREADS, MINB>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, smem);
  return occ;
}

template <bool GB, bool ER>
static int cta_occupancy(int minb, int block, size_t smem) {
  constexpr int LT = GB ? CTA_GB_THREADS : CTA_THREADS;
  return minb >= CTA_MINB_THROUGHPUT
             ? cta_occupancy<GB, ER, CTA_TPUT_THREADS, CTA_MINB_THROUGHPUT>(block, smem)
             : cta_occupancy<GB, ER, LT, CTA_MINB_LATENCY>(block, smem);
}

template <int CL, bool ER>
static void* cta_cluster_fn() {
  return (void*)cta_cluster_kernel<CL, ER>;
}

static void* cluster_kernel(int cl, bool er) {
  switch (cl) {
    case 2: return er ? cta_cluster_fn<2, true>() : cta_cluster_fn<2, false>();
    case 4: return er ? cta_cluster_fn<4, true>() : cta_cluster_fn<4, false>();
    case 8: return er ? cta_cluster_fn<8, true>() : cta_cluster_fn<8, false>();
    default: return nullptr;
  }
}

// Clusters that can be resident at once for a cluster launch of `cl` blocks
// with `smem` bytes of dynamic shared memory each (0 if it cannot launch).
static int cluster_capacity(int cl, bool er, size_t smem, int block) {
  void* fn = cluster_kernel(cl, er);
  if (!fn) return 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(cl);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr{};
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = cl;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// Cluster mode for a call of few sources: the smallest cluster whose slices
// hold the bitmap next to rank 0's queue halves. MSBFS_CTA_CLUSTER=0 turns
// it off, =1 uses it whatever the number of sources.
static bool cta_cluster_shape(uint32_t V, int sms, int optin, bool edge_records,
                              size_t num_sources, CtaShape* out) {
  const char* env = getenv("MSBFS_CTA_CLUSTER");
  const int mode = env ? atoi(env) : -1;
  if (mode == 0) return false;
  const size_t words = ((size_t)V + 31) / 32;
  const size_t entry = edge_records ? 2 * sizeof(uint32_t) : sizeof(uint32_t);
  const size_t slack = 2048;
  for (int cl : {2, 4, 8}) {
    const size_t wpb = (words + cl - 1) / cl;
    const size_t slice = (wpb + 1) / 2 * 2 * sizeof(uint32_t);
    if (slice + 2 * 1024 * entry + slack > (size_t)optin) continue;
    const size_t room = (size_t)optin - slack - slice;
    CtaShape sh{};
    sh.block = CTA_CLUSTER_THREADS;
    sh.edge_records = edge_records;
    sh.cluster = cl;
    sh.minb = 1;
    sh.qh = (uint32_t)std::min<size_t>(CTA_SMEM_QUEUE, room / (2 * entry) / 32 * 32);
    sh.smem = slice + 2 * (size_t)sh.qh * entry;
    const int n = cluster_capacity(cl, edge_records, sh.smem, sh.block);
    if (n < 1) continue;
    // A cluster traverses a source faster than a global-bitmap block, but a
    // global-bitmap launch keeps several blocks per SM busy: clusters pay
    // off while every source has a cluster of its own (road 1448 x 1448:
    // S=64 10.7 vs 18.8 ms; S=152, two sources per cluster, 21.2 vs 22.1;
    // S=256 46.3 vs 28.0 with a 512-thread rank 0).
    if (mode != 1 && num_sources > (size_t)n) return false;
    sh.grid = n * cl;
    (void)sms;
    *out = sh;
    return true;
  }
  return false;
}

bool cta_launch_shape(uint32_t V, int device, bool allow_global, bool edge_records,
                      size_t num_sources, CtaShape* out) {
  int sms = 0, optin = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
  const size_t words = ((size_t)V + 31) / 32;
  const size_t entry = edge_records ? 2 * sizeof(uint32_t) : sizeof(uint32_t);
  const bool shared_bits = (size_t)V <= cta_max_vertices(device);
  if (!shared_bits && !allow_global) return false;
  if (!shared_bits && cta_cluster_shape(V, sms, optin, edge_records, num_sources, out))
    return true;
  CtaShape sh{};
  sh.edge_records = edge_records;
  sh.global_bits = !shared_bits;
  sh.minb = (shared_bits && num_sources > (size_t)sms * CTA_MINB_LATENCY) ? CTA_MINB_THROUGHPUT
                                                                          : CTA_MINB_LATENCY;
  sh.block = sh.minb >= CTA_MINB_THROUGHPUT ? CTA_TPUT_THREADS
             : shared_bits                    ? CTA_THREADS
                                              : CTA_GB_THREADS;
  // The queue halves get the shared memory left once the bitmaps of minb
  // resident blocks have theirs, so the queue never costs a resident block.
  // A frontier beyond the halves continues in the global slab.
  const size_t bitmap = shared_bits ? (words + 1) / 2 * 2 * sizeof(uint32_t) : 0;  // 8-byte end
  const size_t slack = 2048;  // static shared variables + the driver's per-block reserve
  const size_t fit = std::max<size_t>(1, (size_t)per_sm / (bitmap + slack));
  const size_t blocks = std::min<size_t>((size_t)sh.minb, fit);
  const size_t budget = std::min<size_t>((size_t)per_sm / blocks, (size_t)optin) - slack;
  const size_t room = budget > bitmap ? budget - bitmap : 0;
  sh.qh = (uint32_t)std::min<size_t>(CTA_SMEM_QUEUE, room / (2 * entry) / 32 * 32);
  sh.smem = bitmap + 2 * (size_t)sh.qh * entry;
  int occ;
  if (shared_bits)
    occ = edge_records ? cta_occupancy<false, true>(sh.minb, sh.block, sh.smem)
                       : cta_occupancy<false, false>(sh.minb, sh.block, sh.smem);
  else
    occ = edge_records ? cta_occupancy<true, true>(sh.minb, sh.block, sh.smem)
                       : cta_occupancy<true, false>(sh.minb, sh.block, sh.smem);
  if (occ < 1) return false;
  sh.grid = sms * occ;
  if (!shared_bits) {
    const size_t per_block = ((size_t)V + words) * sizeof(uint32_t);
    sh.grid = (int)std::max<size_t>(
        1, std::min<size_t>((size_t)sh.grid, CTA_GLOBAL_SCRATCH_BYTES / per_block));
  }
  *out = sh;
  return true;
}

template <bool GB, bool ER>
static void launch_cta_t(const CtaParams& p, const CtaShape& sh, int grid, cudaStream_t s) {
  constexpr int LT = GB ? CTA_GB_THREADS : CTA_THREADS;
  if (sh.minb >= CTA_MINB_THROUGHPUT)
    cta_bfs_kernel<GB, ER, CTA_TPUT_THREADS, CTA_MINB_THROUGHPUT>
        <<<grid, sh.block, sh.smem, s>>>(p);
  else
    cta_bfs_kernel<GB, ER, LT, CTA_MINB_LATENCY><<<grid, sh.block, sh.smem, s>>>(p);
}

void launch_cta(const CtaParams& params, const CtaShape& sh, int grid, cudaStream_t s) {
  CtaParams p = params;
  p.qh = sh.qh;  // the dynamic shared memory holds exactly these queue halves
  if (!sh.edge_records) p.erec = nullptr;
  if (sh.cluster > 1) {
    // grid: blocks, a multiple of the cluster size (checked by the caller)
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(sh.block);
    cfg.dynamicSmemBytes = sh.smem;
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = sh.cluster;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    void* args[] = {&p};
    cudaLaunchKernelExC(&cfg, cluster_kernel(sh.cluster, sh.edge_records), args);
    return;
  }
  if (sh.global_bits) {
    if (sh.edge_records)
      launch_cta_t<true, true>(p, sh, grid, s);
    else
      launch_cta_t<true, false>(p, sh, grid, s);
  } else {
    if (sh.edge_records)
      launch_cta_t<false, true>(p, sh, grid, s);
    else
      launch_cta_t<false, false>(p, sh, grid, s);
  }
}

// ---------------------------------------------------------------------------
// Allocation-free form of the CTA-per-source launch.
//
// Its scratch -- a copy of the sources, the source cursor and one frontier
// queue slab (V words) per resident block -- lives in this fixed array
// instead of engine-owned cudaMalloc memory, so the entry point below never
// allocates. Every GPU that loads the library holds the array until exit.
// Layout in u32 words: [0] source cursor, [NOALLOC_SRC_OFF, +NOALLOC_SRC_CAP)
// sources of the current chunk, [NOALLOC_Q_OFF, end) queue slabs.
constexpr size_t NOALLOC_WORDS = MSBFS_NOALLOC_SCRATCH_BYTES / sizeof(uint32_t);
constexpr size_t NOALLOC_SRC_OFF = 64;
constexpr size_t NOALLOC_SRC_CAP = 65536;
constexpr size_t NOALLOC_Q_OFF = NOALLOC_SRC_OFF + NOALLOC_SRC_CAP;
static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_WORDS];

namespace {
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_addr[64];  // device address of the array, per device
}  // namespace

}  // namespace msbfs

namespace {

// Restores the calling thread's current device when the entry point returns.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
  }
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" int msbfs_run_cta_noalloc(int device, size_t num_vertices,
                                     const uint32_t* row_offsets_device,
                                     const uint32_t* col_indices_device,
                                     const uint32_t* sources, size_t num_sources,
                                     uint32_t* dist_device, void* cuda_stream) {
  using namespace msbfs;
  if (num_sources == 0) return MSBFS_OK;
  if (device < 0 || device >= 64) return MSBFS_ERR_NO_DEVICE;
  if (!row_offsets_device || !col_indices_device || !sources || !dist_device)
    return MSBFS_ERR_INVALID_ARGUMENT;
  if (num_vertices == 0) return MSBFS_ERR_EMPTY_GRAPH;
  for (size_t i = 0; i < num_sources; ++i)
    if ((size_t)sources[i] >= num_vertices) return MSBFS_ERR_SOURCE_OOB;
  // Size limits, checked before touching the device: the visited bitmap must
  // fit shared memory and at least one queue slab must fit the scratch array.
  if (num_vertices > MSBFS_NOALLOC_MAX_VERTICES ||
      NOALLOC_Q_OFF + num_vertices > NOALLOC_WORDS)
    return MSBFS_ERR_SCRATCH_TOO_SMALL;
  const DeviceRestore restore;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return MSBFS_ERR_NO_DEVICE;
  }
  // Once per device, with that device current: the array's device address
  // (in host code the symbol itself is only a host-side stand-in).
  uint32_t* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return MSBFS_ERR_CUDA;
      }
      g_noalloc_addr[device] = static_cast<uint32_t*>(p);
    }
    base = g_noalloc_addr[device];
  }
  const uint32_t V = (uint32_t)num_vertices;
  CtaShape sh{};
  if (!cta_launch_shape(V, device, /*allow_global=*/false, /*edge_records=*/false, num_sources,
                        &sh))
    return MSBFS_ERR_SCRATCH_TOO_SMALL;
  const size_t slabs = (NOALLOC_WORDS - NOALLOC_Q_OFF) / (size_t)V;
  const cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  // A non-sticky error left on this thread by earlier work would otherwise
  // be reported as this call's launch failure below.
  cudaGetLastError();
  for (size_t s0 = 0; s0 < num_sources; s0 += NOALLOC_SRC_CAP) {
    const size_t n = std::min(NOALLOC_SRC_CAP, num_sources - s0);
    // The cursor must start at zero; queue slabs need no clearing. Chunks
    // follow one another in stream order, so a chunk's copy of its sources
    // cannot overwrite those of the chunk before it while that one runs.
    if (cudaMemsetAsync(base, 0, sizeof(uint32_t), s) != cudaSuccess ||
        cudaMemcpyAsync(base + NOALLOC_SRC_OFF, sources + s0, n * sizeof(uint32_t),
                        cudaMemcpyHostToDevice, s) != cudaSuccess) {
      cudaGetLastError();
      return MSBFS_ERR_CUDA;
    }
    CtaParams cp{};
    cp.V = V;
    cp.off = row_offsets_device;
    cp.idx = col_indices_device;
    cp.sources = base + NOALLOC_SRC_OFF;
    cp.num_sources = (uint32_t)n;
    cp.dist = dist_device + s0 * num_vertices;
    cp.gqueue = base + NOALLOC_Q_OFF;
    cp.work = base;
    const int blocks = (int)std::min<size_t>({(size_t)sh.grid, n, slabs});
    launch_cta(cp, sh, blocks, s);
    if (cudaGetLastError() != cudaSuccess) return MSBFS_ERR_CUDA;
  }
  return MSBFS_OK;
}
