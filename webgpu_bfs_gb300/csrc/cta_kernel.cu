// One-CTA-per-source persistent BFS for low-degree, high-diameter graphs
// (road networks, grids, trees).
//
// Semantics follow crates/shaders/src/workgroup_persistent_bfs.wgsl:62-196
// and crates/gpu_bfs/src/dispatch/workgroup_persistent.rs:288-370 of the
// reference: one workgroup runs a whole single-source BFS with its visited
// bitmap in shared memory and synchronises only inside the block, so a
// ~1,000-level traversal needs no grid-wide step. The GB300 form differs:
// the bitmap takes up to ~200 KB of shared memory (vs 14 KB), the frontier
// queues live in an L2-resident global slab per resident block (no overflow
// fallback), distances are exact u32 written into the caller's row, and the
// grid is persistent: each resident block pulls the next source from an
// atomic cursor until all sources are done. No block ever waits on another.
#include <algorithm>
#include <mutex>

#include "../../include/msbfs.h"
#include "device_common.cuh"

namespace msbfs {

constexpr uint32_t CTA_DIST_MAX = 0xffffffffu;

__global__ void cta_bfs_kernel(CtaParams p) {
  extern __shared__ uint32_t bitmap[];
  __shared__ uint32_t s_src_idx;
  __shared__ uint32_t s_count;
  __shared__ unsigned long long s_sum;
  __shared__ uint32_t s_reached;
  const uint32_t V = p.V;
  const uint32_t words = (V + 31) / 32;
  uint32_t* qa = p.gqueue + (size_t)blockIdx.x * 2 * V;
  uint32_t* qb = qa + V;

  for (;;) {
    if (threadIdx.x == 0) {
      s_src_idx = atomicAdd(p.work, 1u);
      s_sum = 0;
      s_reached = 0;
    }
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) bitmap[i] = 0;
    __syncthreads();
    const uint32_t si = s_src_idx;
    if (si >= p.num_sources) break;
    const uint32_t src = p.sources[si];
    uint32_t* row = p.dist ? p.dist + (size_t)si * V : nullptr;
    if (threadIdx.x == 0) {
      bitmap[src >> 5] = 1u << (src & 31);
      if (row) row[src] = 0;
      qa[0] = src;
      s_count = 0;
    }
    uint32_t n_in = 1;
    uint32_t level = 0, ecc = 0;
    unsigned long long my_sum = 0;
    uint32_t my_cnt = 0;
    uint32_t* qin = qa;
    uint32_t* qout = qb;
    __syncthreads();
    while (n_in) {
      ecc = level;
      const uint32_t nd = level + 1;
      // Threads sweep the frontier; each expands one vertex's out-edges.
      const uint32_t n_round = (n_in + blockDim.x - 1) / blockDim.x * blockDim.x;
      for (uint32_t i = threadIdx.x; i < n_round; i += blockDim.x) {
        if (i < n_in) {
          const uint32_t u = qin[i];
          const uint32_t eb = __ldg(p.off + u), ee = __ldg(p.off + u + 1);
          for (uint32_t e = eb; e < ee; ++e) {
            const uint32_t v = __ldg(p.idx + e);
            const uint32_t bit = 1u << (v & 31);
            if (bitmap[v >> 5] & bit) continue;
            const uint32_t old = atomicOr(&bitmap[v >> 5], bit);
            if (old & bit) continue;
            if (row) row[v] = nd;
            my_sum += nd;
            ++my_cnt;
            const uint32_t pos = atomicAdd(&s_count, 1u);
            qout[pos] = v;
          }
        }
      }
      __syncthreads();
      n_in = s_count;
      __syncthreads();
      if (threadIdx.x == 0) s_count = 0;
      uint32_t* t = qin;
      qin = qout;
      qout = t;
      ++level;
      __syncthreads();
    }
    if (row) {
      // Unreached vertices: coalesced sweep of the row guided by the bitmap.
      for (uint32_t v = threadIdx.x; v < V; v += blockDim.x)
        if (!((bitmap[v >> 5] >> (v & 31)) & 1u)) row[v] = CTA_DIST_MAX;
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

bool cta_launch_shape(uint32_t V, int device, int* grid, int* block, size_t* smem) {
  if ((size_t)V > cta_max_vertices(device)) return false;
  const size_t bytes = ((size_t)V + 31) / 32 * sizeof(uint32_t);
  const int threads = 256;
  cudaFuncSetAttribute(cta_bfs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cta_bfs_kernel, threads, bytes);
  if (occ < 1) return false;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  *grid = sms * occ;
  *block = threads;
  *smem = bytes;
  return true;
}

void launch_cta(const CtaParams& p, int grid, int block, size_t smem, cudaStream_t s) {
  cta_bfs_kernel<<<grid, block, smem, s>>>(p);
}

// ---------------------------------------------------------------------------
// Allocation-free form of the CTA-per-source launch.
//
// Its scratch -- a copy of the sources, the source cursor and one frontier
// queue slab (2*V words) per resident block -- lives in this fixed array
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
      NOALLOC_Q_OFF + 2 * num_vertices > NOALLOC_WORDS)
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
  int grid = 0, block = 0;
  size_t smem = 0;
  if (!cta_launch_shape(V, device, &grid, &block, &smem)) return MSBFS_ERR_SCRATCH_TOO_SMALL;
  const size_t slabs = (NOALLOC_WORDS - NOALLOC_Q_OFF) / (2 * (size_t)V);
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
    const int blocks = (int)std::min<size_t>({(size_t)grid, n, slabs});
    launch_cta(cp, blocks, block, smem, s);
    if (cudaGetLastError() != cudaSuccess) return MSBFS_ERR_CUDA;
  }
  return MSBFS_OK;
}
