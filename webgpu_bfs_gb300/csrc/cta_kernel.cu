// One-CTA-per-source persistent BFS for low-degree, high-diameter graphs
// (road networks, grids, trees).
//
// Semantics follow crates/shaders/src/workgroup_persistent_bfs.wgsl:62-196
// and crates/gpu_bfs/src/dispatch/workgroup_persistent.rs:288-370 of the
// reference: one workgroup runs a whole single-source BFS with its visited
// bitmap in shared memory and synchronises only inside the block, so a
// ~1,000-level traversal needs no grid-wide step. The GB300 form differs:
// the bitmap takes up to ~227 KB of shared memory (vs 14 KB) and, for larger
// graphs, moves to an L2-resident global slab per block instead of giving up
// the path; the frontier queues live in one L2-resident global slab of V
// words per resident block (no overflow fallback), distances are exact u32
// written into the caller's row, and the grid is persistent: each resident
// block pulls the next source from an atomic cursor until all sources are
// done. No block ever waits on another.
#include <algorithm>
#include <mutex>

#include "../../include/msbfs.h"
#include "device_common.cuh"

namespace msbfs {

constexpr uint32_t CTA_DIST_MAX = 0xffffffffu;
constexpr int CTA_THREADS = 512;
// Global-bitmap mode keeps its per-block scratch (queue slab + bitmap) within
// this many bytes by shrinking the grid.
constexpr size_t CTA_GLOBAL_SCRATCH_BYTES = 4ull << 30;

// GB: the visited bitmap lives in an L2-resident global slab per block (for
// graphs whose bitmap does not fit shared memory) instead of shared memory.
//
// Queue: one slab of V words per block. The frontiers of consecutive levels
// are disjoint vertex sets, so |F_L| + |F_L+1| <= V: even levels read from
// the front of the slab and append at the back, odd levels the reverse.
// Counters: level L appends through s_cnt[L % 3]; thread 0 clears
// s_cnt[(L+1) % 3] during level L (last read right after the barrier of
// level L-2), so a level needs one block barrier.
template <bool GB>
__global__ void __launch_bounds__(CTA_THREADS) cta_bfs_kernel(CtaParams p) {
  extern __shared__ uint32_t smem_bits[];
  __shared__ uint32_t s_src_idx;
  __shared__ uint32_t s_cnt[3];
  __shared__ unsigned long long s_sum;
  __shared__ uint32_t s_reached;
  const uint32_t V = p.V;
  const uint32_t words = (V + 31) / 32;
  uint32_t* bits = GB ? p.gbits + (size_t)blockIdx.x * words : smem_bits;
  uint32_t* slab = p.gqueue + (size_t)blockIdx.x * V;

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
      slab[0] = src;
    }
    uint32_t n_in = 1;
    uint32_t level = 0, ecc = 0;
    unsigned long long my_sum = 0;
    uint32_t my_cnt = 0;
    __syncthreads();
    while (n_in) {
      ecc = level;
      const uint32_t nd = level + 1;
      const bool front = (level & 1) == 0;  // where this level's frontier sits
      uint32_t* cnt = &s_cnt[level % 3];
      if (threadIdx.x == 0) s_cnt[(level + 1) % 3] = 0;
      // Threads sweep the frontier; each expands one vertex's out-edges.
      for (uint32_t i = threadIdx.x; i < n_in; i += blockDim.x) {
        const uint32_t u = front ? slab[i] : slab[V - 1 - i];
        const uint32_t eb = __ldg(p.off + u), ee = __ldg(p.off + u + 1);
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
          const uint32_t pos = atomicAdd(cnt, 1u);
          if (front)
            slab[V - 1 - pos] = v;
          else
            slab[pos] = v;
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

size_t cta_max_vertices(int device) {
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  const size_t reserve = 1024;  // static shared variables and slack
  if (optin <= (int)reserve) return 0;
  return ((size_t)optin - reserve) * 8;
}

bool cta_launch_shape(uint32_t V, int device, bool allow_global, CtaShape* out) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const size_t words = ((size_t)V + 31) / 32;
  CtaShape sh{};
  sh.block = CTA_THREADS;
  int occ = 0;
  if ((size_t)V <= cta_max_vertices(device)) {
    sh.smem = words * sizeof(uint32_t);
    cudaFuncSetAttribute(cta_bfs_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sh.smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cta_bfs_kernel<false>, sh.block,
                                                  sh.smem);
    if (occ < 1) return false;
    sh.grid = sms * occ;
  } else {
    if (!allow_global) return false;
    sh.global_bits = true;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cta_bfs_kernel<true>, sh.block, 0);
    if (occ < 1) return false;
    const size_t per_block = ((size_t)V + words) * sizeof(uint32_t);
    sh.grid = (int)std::max<size_t>(
        1, std::min<size_t>((size_t)sms * occ, CTA_GLOBAL_SCRATCH_BYTES / per_block));
  }
  *out = sh;
  return true;
}

void launch_cta(const CtaParams& p, const CtaShape& sh, int grid, cudaStream_t s) {
  if (sh.global_bits)
    cta_bfs_kernel<true><<<grid, sh.block, 0, s>>>(p);
  else
    cta_bfs_kernel<false><<<grid, sh.block, sh.smem, s>>>(p);
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
  if (!cta_launch_shape(V, device, /*allow_global=*/false, &sh))
    return MSBFS_ERR_SCRATCH_TOO_SMALL;
  const size_t slabs = (NOALLOC_WORDS - NOALLOC_Q_OFF) / (size_t)V;
  const cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  for (size_t s0 = 0; s0 < num_sources; s0 += NOALLOC_SRC_CAP) {
    const size_t n = std::min(NOALLOC_SRC_CAP, num_sources - s0);
    // The cursor must start at zero; queue slabs need no clearing.
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
