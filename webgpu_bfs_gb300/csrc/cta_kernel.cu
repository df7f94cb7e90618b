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
#include "device_common.cuh"

namespace msbfs {

constexpr uint32_t CTA_DIST_MAX = 0xffffffffu;

__global__ void cta_bfs_kernel(CtaParams p) {
  extern __shared__ uint32_t bitmap[];
  __shared__ uint32_t s_src_idx;
  __shared__ uint32_t s_count;
  const uint32_t V = p.V;
  const uint32_t words = (V + 31) / 32;
  const uint32_t lane = threadIdx.x & 31;
  uint32_t* qa = p.gqueue + (size_t)blockIdx.x * 2 * V;
  uint32_t* qb = qa + V;

  for (;;) {
    if (threadIdx.x == 0) s_src_idx = atomicAdd(p.work, 1u);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) bitmap[i] = 0;
    __syncthreads();
    const uint32_t si = s_src_idx;
    if (si >= p.num_sources) break;
    const uint32_t src = p.sources[si];
    uint32_t* row = p.dist + (size_t)si * V;
    if (threadIdx.x == 0) {
      bitmap[src >> 5] = 1u << (src & 31);
      row[src] = 0;
      qa[0] = src;
      s_count = 0;
    }
    uint32_t n_in = 1;
    uint32_t level = 0;
    uint32_t* qin = qa;
    uint32_t* qout = qb;
    __syncthreads();
    while (n_in) {
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
            row[v] = nd;
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
    // Unreached vertices: coalesced sweep of the row guided by the bitmap.
    for (uint32_t v = threadIdx.x; v < V; v += blockDim.x)
      if (!((bitmap[v >> 5] >> (v & 31)) & 1u)) row[v] = CTA_DIST_MAX;
    (void)lane;
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

}  // namespace msbfs
