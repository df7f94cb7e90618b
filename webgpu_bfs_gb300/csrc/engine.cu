// Engine: the C ABI of include/msbfs.h over the sm_103a kernels.
//
// Mirrors crates/gpu_bfs/src/engine.rs of the reference (GpuBfsEngine: method
// enum, Auto router, per-call source validation, pooled device buffers behind
// a mutex) with a CUDA runtime underneath instead of wgpu:
//  * graphs are uploaded once and stay resident (CSR + CSC, aliased when the
//    graph is symmetric, like PushPullGraphBuffers in buffer.rs:108-221);
//  * a level-synchronous pass is ONE cudaGraphLaunch: memset control block,
//    source init, a WHILE conditional node around the level kernel (its last
//    block sets the condition, so no host round trip per level or per batch
//    of levels, replacing multi_word_bp.rs:730-814's speculative 4..64-hop
//    submits and indirect_sparse_push.rs:1462-1578's macro batches), the
//    distance materialisation and the frontier cleanup;
//  * the CTA-per-source path is one persistent launch per call.
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/msbfs.h"
#include "device_common.cuh"
#include "host_graph.h"

using namespace msbfs;

#ifndef MSBFS_PUSH_SEG
#define MSBFS_PUSH_SEG 64
#endif
#ifndef MSBFS_PUSH_SEG0
#define MSBFS_PUSH_SEG0 8  // out-edges per entry of the sources' queue
#endif

namespace {

struct Workspace;

}  // namespace

struct msbfs_graph {
  msbfs_engine* eng = nullptr;
  std::vector<msbfs_engine*> users;  // other engines of the device that may run on it
  uint64_t id = 0;  // unique in the process: keys every engine's workspaces
  size_t V = 0, E = 0;
  bool sym = false;
  uint32_t max_deg = 0;
  uint32_t* off = nullptr;   // CSR
  uint32_t* idx = nullptr;
  uint32_t* coff = nullptr;  // CSC (== CSR when symmetric)
  uint32_t* cidx = nullptr;
  // In-edge lists longer than `split` are cut into slices for bottom-up steps.
  uint32_t split = 0;
  uint32_t n_heavy = 0;
  uint32_t n_hchunks = 0;
  HeavyChunk* hchunks = nullptr;
  // Bottom-up work order: vertices with 0 < in-degree <= split, ascending ids.
  uint32_t n_order = 0;
  uint4* order = nullptr;  // {vertex, in-edge begin, in-edge end, 0}
  // Road-like graphs: per edge {target, target's edge begin, end, 0}.
  uint4* erec = nullptr;
  std::vector<uint32_t> h_coff;  // host CSC offsets (V + 1): rebuilds the tables above
};

namespace {

struct Workspace {
  uint64_t graph_id = 0;
  uint32_t W = 0;
  uint32_t mode = 0;
  bool count = false;  // level kernels keep the profiling counters
  LevelParams p{};
  LevelKernelInfo k{};
  LevelCtl* d_ctl = nullptr;
  PassDesc* d_desc = nullptr;
  LevelRec* d_log = nullptr;
  std::vector<void*> allocs;
  // Set when a pass stopped part-way (an error after work was queued): its
  // buffers may hold that pass's bits, so the next call builds a fresh
  // workspace instead of reusing this one.
  bool dirty = false;
  // One instantiated pass per ending: [0] materialise, [1] reduce, [2] the
  // byte rows of a split materialisation only (built on first use).
  cudaGraph_t graph[3] = {nullptr, nullptr, nullptr};
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
  ~Workspace() {
    for (int i = 0; i < 3; ++i) {
      if (exec[i]) cudaGraphExecDestroy(exec[i]);
      if (graph[i]) cudaGraphDestroy(graph[i]);
    }
    for (void* a : allocs) cudaFree(a);
  }
};

uint32_t bit_length_u64(uint64_t x) {
  uint32_t n = 0;
  while (x) {
    ++n;
    x >>= 1;
  }
  return n;
}

uint32_t method_path(int m) {
  switch (m) {
    case MSBFS_METHOD_WORKGROUP_PERSISTENT_BFS:
      return MSBFS_PATH_CTA;
    case MSBFS_METHOD_MULTI_WORD_BIT_PARALLEL:
    case MSBFS_METHOD_BIT_PARALLEL_64_PULL:
    case MSBFS_METHOD_INDIRECT_MACRO_BATCH:
      return MSBFS_PATH_PULL;
    case MSBFS_METHOD_BIT_PARALLEL_32:
    case MSBFS_METHOD_BIT_PARALLEL_64:
    case MSBFS_METHOD_SPARSE_BIT_PARALLEL_64:
    case MSBFS_METHOD_MULTI_WORD_BIT_PARALLEL_PUSH:
    case MSBFS_METHOD_BOOLEAN_REACHABILITY:
      return MSBFS_PATH_PUSH;
    default:
      return MSBFS_PATH_HYBRID;
  }
}

}  // namespace

struct msbfs_engine {
  int device = 0;
  int method = MSBFS_METHOD_AUTO;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_pass = nullptr, ev_copies = nullptr;
  std::mutex mu;
  std::string last_error;
  uint32_t max_words = 16;
  uint32_t alpha = 14;
  uint32_t beta = 24;
  uint32_t seg = MSBFS_PUSH_SEG;  // out-edges per top-down queue entry
#ifndef MSBFS_HEAVY
#define MSBFS_HEAVY 32
#endif
  uint32_t heavy = MSBFS_HEAVY;  // in-degree from which a whole warp scans a vertex
#ifndef MSBFS_SPLIT
// At 8 resident level blocks per SM (R-MAT scale 22, S=512, 2 tiles per
// claim): 512 8.59 ms per step, 384 8.73, 640 8.53, 1,024 9.67, 256 9.41.
#define MSBFS_SPLIT 512
#endif
  uint32_t split = MSBFS_SPLIT;  // in-edge slice length of bottom-up steps
  uint32_t bits_div = 64;
  uint32_t sm_share = 100;  // percent of the resident grid the persistent kernels use
#ifndef MSBFS_MAT_WAVES
// R-MAT scale 22, S=512, materialisation ms: 1 wave (persistent) 1.82, 2
// 1.81, 4 1.69, 8 1.65, one block per tile 1.59. Blocks of a long
// grid-stride loop drift apart and spread their row writes over more DRAM
// pages; a write-only kernel with the same 256-byte row segments reaches
// 6.5 TB/s persistent at 5 blocks per SM and 7.4 TB/s in short blocks.
#define MSBFS_MAT_WAVES 0
#endif
  // Materialisation grid in waves of its resident blocks (0: one block per
  // tile); a smaller SM share keeps it persistent at that share.
  uint32_t mat_waves = MSBFS_MAT_WAVES;
  uint32_t level_cap = 0;   // levels per pass before MSBFS_ERR_TIMEOUT (0: V + 2)
  bool host_loop = false;
  bool zero_copy = true;  // MSBFS_ZERO_COPY=0 stages host output in HBM instead
  bool narrow = true;     // MSBFS_NARROW=0 keeps host-bound rows u32 over the link
  int profiling = 0;
  std::vector<msbfs_level_record> log;       // records of the last call
  LevelRec* h_log = nullptr;                 // pinned, LOG_CAP per pass
  size_t h_log_passes = 0;
  std::vector<cudaEvent_t> lvl_events;       // profiling levels 2 and 3
  std::vector<std::vector<float>> pass_event_ms;
  std::map<std::tuple<uint64_t, uint32_t, uint32_t>, std::unique_ptr<Workspace>> ws;
  // call scratch
  uint32_t* d_sources = nullptr;
  size_t d_sources_cap = 0;
  uint32_t* d_dist = nullptr;
  size_t d_dist_cap = 0;  // u32 elements
  uint8_t* d_dist8 = nullptr;  // byte rows of host-bound calls
  size_t d_dist8_cap = 0;
  uint8_t* h_dist8 = nullptr;  // page-locked landing buffer of the byte rows
  size_t h_dist8_cap = 0;
  std::vector<cudaEvent_t> chunk_events;  // one per landed chunk of byte rows
  // Page-locked output: share of a pass's rows written as u32 over the link
  // (MSBFS_SPLIT_ROWS; R-MAT 22, S=512: 1.0 50.5 ms per call, 0.8 47.0,
  // 0.7 45.8, 0.6 44.0, 0.5 ~45).
  double split_frac = 0.6;
  bool last_split = false;   // the last call split its materialisation
  std::vector<uint32_t> split_rows;         // per pass: first byte row
  std::vector<cudaEvent_t> split_events;    // per pass: its byte rows are done
  uint32_t* d_reach = nullptr;
  size_t d_reach_cap = 0;
  uint32_t* d_cta_queue = nullptr;
  size_t d_cta_queue_cap = 0;
  uint32_t* d_cta_bits = nullptr;  // global-bitmap mode of the CTA path
  size_t d_cta_bits_cap = 0;
  uint32_t* d_work = nullptr;
  unsigned long long* d_counter = nullptr;
  SourceStats* d_sstats = nullptr;  // per-source reductions of host-output calls
  size_t d_sstats_cap = 0;
  LevelCtl* h_ctl = nullptr;  // pinned, one per pass of the last call
  size_t h_ctl_cap = 0;
  // last call
  msbfs_stats last{};
  size_t last_passes = 0;
  bool last_level_path = false;
};

namespace {

int set_err(msbfs_engine* e, int code, const std::string& msg) {
  if (e) e->last_error = msg;
  return code;
}

int cuda_fail(msbfs_engine* e, cudaError_t err, const char* what) {
  cudaGetLastError();  // clear sticky-free errors
  std::string m = std::string(what) + ": " + cudaGetErrorString(err);
  return set_err(e, err == cudaErrorMemoryAllocation ? MSBFS_ERR_OOM : MSBFS_ERR_CUDA, m);
}

#define CK(call)                                            \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return cuda_fail(eng, _e, #call); \
  } while (0)

template <typename T>
int grow(msbfs_engine* eng, T** ptr, size_t* cap, size_t need) {
  if (need <= *cap && *ptr) return MSBFS_OK;
  if (*ptr) {
    // Earlier asynchronous calls may still read the old buffer.
    CK(cudaStreamSynchronize(eng->stream));
    CK(cudaStreamSynchronize(eng->copy_stream));
    cudaFree(*ptr);
  }
  *ptr = nullptr;
  *cap = 0;
  size_t n = std::max(need, (size_t)1);
  CK(cudaMalloc((void**)ptr, n * sizeof(T)));
  *cap = n;
  return MSBFS_OK;
}

int dev_alloc(msbfs_engine* eng, Workspace* w, void** ptr, size_t bytes) {
  if (bytes == 0) bytes = 16;
  CK(cudaMalloc(ptr, bytes));
  w->allocs.push_back(*ptr);
  CK(cudaMemsetAsync(*ptr, 0, bytes, eng->stream));
  return MSBFS_OK;
}

// The pass ends in materialize_kernel (variant 0), reduce_kernel (1,
// per-source reductions) or, for a split materialisation, the byte-row
// phase alone (2: the host then launches the u32 phase and the cleanup).
enum : int { PASS_ROWS = 0, PASS_STATS = 1, PASS_BYTES = 2 };
int build_graph_exec(msbfs_engine* eng, Workspace* w, int variant) {
  const bool reduce = variant == PASS_STATS;
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  w->graph[variant] = g;
  cudaGraphNode_t n_mctl, n_mst, n_init, n_cond, n_lvl, n_mat, n_clean;
  cudaMemsetParams m1{};
  m1.dst = w->d_ctl;
  m1.value = 0;
  m1.elementSize = 1;
  m1.width = sizeof(LevelCtl);
  m1.height = 1;
  m1.pitch = sizeof(LevelCtl);
  CK(cudaGraphAddMemsetNode(&n_mctl, g, nullptr, 0, &m1));
  cudaMemsetParams m2{};
  m2.dst = w->p.stamp;
  m2.value = 0xFFFFFFFFu;
  m2.elementSize = 4;
  m2.width = w->p.V;
  m2.height = 1;
  m2.pitch = (size_t)w->p.V * 4;
  CK(cudaGraphAddMemsetNode(&n_mst, g, nullptr, 0, &m2));
  cudaGraphNode_t n_mfb;
  cudaMemsetParams m3{};
  m3.dst = w->p.fbits[0];
  m3.value = 0;
  m3.elementSize = 4;
  m3.width = 3 * (((size_t)w->p.V + 31) / 32);
  m3.height = 1;
  m3.pitch = m3.width * 4;
  CK(cudaGraphAddMemsetNode(&n_mfb, g, nullptr, 0, &m3));
  cudaGraphNode_t n_mhl;
  cudaMemsetParams m4{};
  m4.dst = w->p.hlive;
  m4.value = 0xFFFFFFFFu;
  m4.elementSize = 4;
  m4.width = std::max(w->p.hlive_words, 1u);
  m4.height = 1;
  m4.pitch = m4.width * 4;
  CK(cudaGraphAddMemsetNode(&n_mhl, g, nullptr, 0, &m4));

  void* args_p[] = {&w->p};
  cudaKernelNodeParams ki{};
  ki.func = w->k.init;
  ki.gridDim = dim3(1);
  ki.blockDim = dim3(256);
  ki.sharedMemBytes = 0;
  ki.kernelParams = args_p;
  cudaGraphNode_t deps_init[4] = {n_mctl, n_mst, n_mfb, n_mhl};
  CK(cudaGraphAddKernelNode(&n_init, g, deps_init, 4, &ki));

  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  CK(cudaGraphAddNode(&n_cond, g, &n_init, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];

  // Loop body: the bottom-up kernel, then the top-down kernel; the one whose
  // direction the control block does not name returns at once (a mode
  // that never changes direction gets only its own).
  void* args_l[] = {&w->p, &h};
  n_lvl = nullptr;
  for (uint32_t dir : {(uint32_t)DIR_PULL, (uint32_t)DIR_PUSH}) {
    if ((dir == DIR_PULL && w->mode == MODE_PUSH) || (dir == DIR_PUSH && w->mode == MODE_PULL))
      continue;
    cudaKernelNodeParams kl{};
    kl.func = w->k.level[dir][w->count];
    kl.gridDim = dim3(w->k.level_grids[dir]);
    kl.blockDim = dim3(w->k.level_block);
    kl.sharedMemBytes = 0;
    kl.kernelParams = args_l;
    cudaGraphNode_t prev = n_lvl;
    CK(cudaGraphAddKernelNode(&n_lvl, body, prev ? &prev : nullptr, prev ? 1 : 0, &kl));
  }

  uint32_t phase = variant == PASS_BYTES ? MAT_BYTES : MAT_ALL;
  void* args_m[] = {&w->p, &phase};
  cudaKernelNodeParams km{};
  km.func = reduce ? w->k.reduce : w->k.materialize;
  km.gridDim = dim3(reduce ? w->k.red_grid : w->k.mat_grid);
  km.blockDim = dim3(reduce ? w->k.red_block : w->k.mat_block);
  km.sharedMemBytes = reduce ? 0u : (unsigned)w->k.mat_smem;
  km.kernelParams = reduce ? args_p : args_m;
  CK(cudaGraphAddKernelNode(&n_mat, g, &n_cond, 1, &km));

  if (variant != PASS_BYTES) {
    cudaKernelNodeParams kc{};
    kc.func = w->k.cleanup;
    kc.gridDim = dim3(256);
    kc.blockDim = dim3(256);
    kc.sharedMemBytes = 0;
    kc.kernelParams = args_p;
    CK(cudaGraphAddKernelNode(&n_clean, g, &n_cond, 1, &kc));
  }
  (void)n_lvl;
  (void)n_mat;
  (void)n_clean;
  CK(cudaGraphInstantiate(&w->exec[variant], g, 0));
  return MSBFS_OK;
}

int get_workspace(msbfs_engine* eng, const msbfs_graph* g, uint32_t W, uint32_t mode,
                  Workspace** out) {
  auto key = std::make_tuple(g->id, W, mode);
  auto it = eng->ws.find(key);
  if (it != eng->ws.end()) {
    if (!it->second->dirty) {
      *out = it->second.get();
      return MSBFS_OK;
    }
    CK(cudaStreamSynchronize(eng->stream));
    CK(cudaStreamSynchronize(eng->copy_stream));
    eng->ws.erase(it);
  }
  // One pooled workspace per graph: drop any other (W, mode) of this graph
  // only if memory runs short (allocation failure below retries once).
  auto w = std::make_unique<Workspace>();
  w->graph_id = g->id;
  w->W = W;
  w->mode = mode;
  const uint32_t dist_bits = bit_length_u64(g->V > 1 ? g->V - 1 : 1);
  const uint32_t NP = std::min<uint32_t>(dist_bits, 8);
  if (!level_kernel_info(W, NP, eng->num_sms, &w->k))
    return set_err(eng, MSBFS_ERR_INVALID_ARGUMENT, "unsupported words per vertex");
  // Work is claimed dynamically, so a smaller grid is only slower, never wrong.
  w->count = eng->profiling == 1 || eng->profiling == 2;
  for (int d = 0; d < 2; ++d)
    w->k.level_grids[d] = std::max(1, (int)((uint64_t)w->k.level_grids[d] * eng->sm_share / 100));
  if (eng->sm_share < 100) {
    w->k.mat_grid = std::max(1, (int)((uint64_t)w->k.mat_grid * eng->sm_share / 100));
  } else {
    const size_t items = materialize_items((uint32_t)g->V, W);
    const size_t want = eng->mat_waves ? (size_t)w->k.mat_grid * eng->mat_waves : items;
    w->k.mat_grid = (int)std::max<size_t>(1, std::min(want, items));
  }
  w->k.red_grid = std::max(1, (int)((uint64_t)w->k.red_grid * eng->sm_share / 100));
  LevelParams& p = w->p;
  p.V = (uint32_t)g->V;
  p.W = W;
  p.E = g->E;
  p.out_off = g->off;
  p.out_idx = g->idx;
  p.in_off = g->coff;
  p.in_idx = g->cidx;
  const size_t VW = g->V * (size_t)W;
  p.NP = NP;
  // A level's queue holds each vertex once (the stamp), so V + E/seg
  // entries bound it; the sources' queue (slot 0 at level 0) uses seg0.
  p.qcap = (uint32_t)std::min<uint64_t>(g->V + g->E / eng->seg + 1, 0xFFFFFFFFull);
  const uint64_t qcap0 = std::min<uint64_t>(g->V + g->E / MSBFS_PUSH_SEG0 + 1, 0xFFFFFFFFull);
  p.qcap0 = (uint32_t)qcap0;
  p.mode = mode;
  p.alpha = eng->alpha;
  p.beta = eng->beta;
  p.seg = eng->seg;
  p.seg0 = std::min<uint32_t>(MSBFS_PUSH_SEG0, eng->seg);
  p.heavy = eng->heavy;
  p.bits_div = eng->bits_div;
  p.max_levels = (uint32_t)std::min<uint64_t>(g->V + 2, 0xFFFFFFF0ull);
  if (eng->level_cap) p.max_levels = std::min(p.max_levels, eng->level_cap);
  p.split = g->split;
  p.n_hchunks = g->n_hchunks;
  p.hchunks = g->hchunks;
  p.n_order = g->n_order;
  p.order = g->order;
  int rc;
  void* ptr;
  if ((rc = dev_alloc(eng, w.get(), &ptr, VW * 4))) return rc;
  p.vis = (uint32_t*)ptr;
  for (int i = 0; i < 3; ++i) {
    if ((rc = dev_alloc(eng, w.get(), &ptr, VW * 4))) return rc;
    p.F[i] = (uint32_t*)ptr;
  }
  if ((rc = dev_alloc(eng, w.get(), &ptr, VW * 4 * (size_t)p.NP))) return rc;
  p.planes = (uint32_t*)ptr;
  if ((rc = dev_alloc(eng, w.get(), &ptr, VW * 4))) return rc;
  p.ovf = (uint32_t*)ptr;
  for (int i = 0; i < 3; ++i) {
    if ((rc = dev_alloc(eng, w.get(), &ptr, (size_t)(i == 0 ? qcap0 : p.qcap) * 8))) return rc;
    p.Q[i] = (unsigned long long*)ptr;
  }
  if ((rc = dev_alloc(eng, w.get(), &ptr, g->V * 4))) return rc;
  p.stamp = (uint32_t*)ptr;
  const size_t fwords = (g->V + 31) / 32;
  if ((rc = dev_alloc(eng, w.get(), &ptr, 3 * fwords * 4))) return rc;
  for (int i = 0; i < 3; ++i) p.fbits[i] = (uint32_t*)ptr + i * fwords;
  if ((rc = dev_alloc(eng, w.get(), &ptr, sizeof(LevelCtl)))) return rc;
  w->d_ctl = (LevelCtl*)ptr;
  p.ctl = w->d_ctl;
  if ((rc = dev_alloc(eng, w.get(), &ptr, sizeof(PassDesc)))) return rc;
  w->d_desc = (PassDesc*)ptr;
  p.desc = w->d_desc;
  if ((rc = dev_alloc(eng, w.get(), &ptr, sizeof(LevelRec) * LOG_CAP))) return rc;
  w->d_log = (LevelRec*)ptr;
  p.log = w->d_log;
  if ((rc = dev_alloc(eng, w.get(), &ptr, (size_t)g->n_heavy * W * 4))) return rc;
  p.hcand = (uint32_t*)ptr;
  if ((rc = dev_alloc(eng, w.get(), &ptr, (size_t)g->n_heavy * 4))) return rc;
  p.hcount = (uint32_t*)ptr;
  p.hlive_words = (g->n_hchunks + 31) / 32;
  if ((rc = dev_alloc(eng, w.get(), &ptr, (size_t)std::max(p.hlive_words, 1u) * 4))) return rc;
  p.hlive = (uint32_t*)ptr;
  if (!eng->host_loop) {
    rc = build_graph_exec(eng, w.get(), PASS_ROWS);
    if (rc) {
      // Conditional graph nodes unavailable: fall back to the host-driven loop.
      eng->host_loop = true;
      cudaGetLastError();
    }
  }
  *out = w.get();
  eng->ws[key] = std::move(w);
  return MSBFS_OK;
}

// Host-driven fallback loop: launches level kernels in speculative batches of
// 8 and reads the control block between batches (extra launches after the
// last level return immediately).
int ensure_events(msbfs_engine* eng, size_t n) {
  while (eng->lvl_events.size() < n) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    eng->lvl_events.push_back(e);
  }
  return MSBFS_OK;
}

// Profiling form of the host-driven loop: one level kernel at a time with a
// CUDA event on each side, then the materialisation likewise. The last entry
// of the returned vector is the materialisation.
int run_pass_profiled(msbfs_engine* eng, Workspace* w, bool reduce, std::vector<float>* ms) {
  int rc;
  CK(cudaMemsetAsync(w->d_ctl, 0, sizeof(LevelCtl), eng->stream));
  CK(cudaMemsetAsync(w->p.stamp, 0xFF, w->p.V * sizeof(uint32_t), eng->stream));
  CK(cudaMemsetAsync(w->p.fbits[0], 0, 3 * ((w->p.V + 31) / 32) * sizeof(uint32_t), eng->stream));
  if (w->p.hlive_words)
    CK(cudaMemsetAsync(w->p.hlive, 0xFF, w->p.hlive_words * sizeof(uint32_t), eng->stream));
  launch_init(w->p, eng->stream);
  LevelCtl probe{};
  CK(cudaMemcpyAsync(&probe, w->d_ctl, sizeof(LevelCtl), cudaMemcpyDeviceToHost, eng->stream));
  CK(cudaStreamSynchronize(eng->stream));
  ms->clear();
  for (uint32_t L = 0;; ++L) {
    if ((rc = ensure_events(eng, 2))) return rc;
    CK(cudaEventRecord(eng->lvl_events[0], eng->stream));
    launch_level(w->p, w->k, probe.dir, w->count, eng->stream);
    CK(cudaEventRecord(eng->lvl_events[1], eng->stream));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&probe, w->d_ctl, sizeof(LevelCtl), cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    float t = 0.f;
    cudaEventElapsedTime(&t, eng->lvl_events[0], eng->lvl_events[1]);
    ms->push_back(t);
    if (probe.terminated) break;
    if (L > w->p.max_levels) {
      w->dirty = true;
      return set_err(eng, MSBFS_ERR_TIMEOUT, "level loop did not terminate");
    }
  }
  CK(cudaEventRecord(eng->lvl_events[0], eng->stream));
  launch_materialize(w->p, w->k, reduce, eng->stream);
  CK(cudaEventRecord(eng->lvl_events[1], eng->stream));
  launch_cleanup(w->p, eng->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(eng->stream));
  float t = 0.f;
  cudaEventElapsedTime(&t, eng->lvl_events[0], eng->lvl_events[1]);
  ms->push_back(t);
  return MSBFS_OK;
}

int run_pass_host_loop(msbfs_engine* eng, Workspace* w, bool reduce) {
  CK(cudaMemsetAsync(w->d_ctl, 0, sizeof(LevelCtl), eng->stream));
  CK(cudaMemsetAsync(w->p.stamp, 0xFF, w->p.V * sizeof(uint32_t), eng->stream));
  CK(cudaMemsetAsync(w->p.fbits[0], 0, 3 * ((w->p.V + 31) / 32) * sizeof(uint32_t), eng->stream));
  if (w->p.hlive_words)
    CK(cudaMemsetAsync(w->p.hlive, 0xFF, w->p.hlive_words * sizeof(uint32_t), eng->stream));
  launch_init(w->p, eng->stream);
  LevelCtl probe{};
  for (uint64_t launched = 0;;) {
    const uint32_t dirs = w->mode == MODE_PUSH ? DIR_PUSH : w->mode == MODE_PULL ? DIR_PULL
                                                                                  : DIR_BOTH;
    for (int i = 0; i < 8; ++i) launch_level(w->p, w->k, dirs, w->count, eng->stream);
    launched += 8;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&probe, w->d_ctl, sizeof(LevelCtl), cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    if (probe.terminated) break;
    if (launched > (uint64_t)w->p.max_levels + 16) {
      w->dirty = true;
      return set_err(eng, MSBFS_ERR_TIMEOUT, "level loop did not terminate");
    }
  }
  launch_materialize(w->p, w->k, reduce, eng->stream);
  launch_cleanup(w->p, eng->stream);
  CK(cudaGetLastError());
  return MSBFS_OK;
}

uint32_t choose_words(msbfs_engine* eng, size_t S) {
  size_t lanes = std::min<size_t>(S, (size_t)eng->max_words * 32);
  uint32_t need = (uint32_t)((lanes + 31) / 32);
  uint32_t W = 1;
  while (W < need) W <<= 1;
  return std::min<uint32_t>(W, 64);
}

int validate_call(msbfs_engine* eng, const msbfs_graph* g, const uint32_t* sources, size_t S) {
  if (!eng) return MSBFS_ERR_INVALID_ARGUMENT;
  if (!g) return set_err(eng, MSBFS_ERR_INVALID_ARGUMENT, "graph is null");
  if (g->eng != eng && std::find(g->users.begin(), g->users.end(), eng) == g->users.end())
    return set_err(eng, MSBFS_ERR_INVALID_ARGUMENT, "graph belongs to another engine");
  if (S == 0) return MSBFS_OK;
  if (!sources) return set_err(eng, MSBFS_ERR_INVALID_ARGUMENT, "sources is null");
  char buf[160];
  if (g->V == 0) {
    snprintf(buf, sizeof buf, "Source vertex %u at index 0 exceeds graph vertex count 0", sources[0]);
    return set_err(eng, MSBFS_ERR_EMPTY_GRAPH, buf);
  }
  for (size_t i = 0; i < S; ++i)
    if ((size_t)sources[i] >= g->V) {
      snprintf(buf, sizeof buf, "Source vertex %u at index %zu exceeds graph vertex count %zu",
               sources[i], i, g->V);
      return set_err(eng, MSBFS_ERR_SOURCE_OOB, buf);
    }
  return MSBFS_OK;
}

// The router's road test (engine.rs:157-198): low degree, sparse.
bool is_road_like(const msbfs_graph* g) { return g->max_deg <= 8 && g->E <= 4 * g->V; }

int resolve_method(const msbfs_graph* g, int method, size_t S) {
  if (method == MSBFS_METHOD_AUTO) {
    if (g->V == 0 || S == 0) return MSBFS_METHOD_NAIVE_SEQUENTIAL;
    if (is_road_like(g)) return MSBFS_METHOD_WORKGROUP_PERSISTENT_BFS;
    if (g->max_deg >= 128) return MSBFS_METHOD_INDIRECT_SPARSE_QUEUE_PUSH;
    if (S >= 64) return MSBFS_METHOD_MULTI_WORD_BIT_PARALLEL;
    if (S >= 32) return MSBFS_METHOD_BIT_PARALLEL_64;
    if (S > 1) return MSBFS_METHOD_BIT_PARALLEL_32;
    return MSBFS_METHOD_SPARSE_QUEUE;
  }
  return method;
}

// Queues a whole call on eng->stream. dist_dev: S*V output (device) or null
// in reachability mode; reach_dev: V*ceil(S/32) words (device) or null.
// host_out / host_reach: when non-null, rows are copied back per pass on the
// copy stream while later passes run.
int enqueue_call(msbfs_engine* eng, int method, const msbfs_graph* g, const uint32_t* sources,
                 size_t S, uint32_t* dist_dev, uint32_t* reach_dev, uint32_t* host_out,
                 uint32_t* host_reach, SourceStats* stats_dev = nullptr,
                 uint8_t* dist8_dev = nullptr, double split_frac = 0.0) {
  int rc;
  if (stats_dev) CK(cudaMemsetAsync(stats_dev, 0, S * sizeof(SourceStats), eng->stream));
  const int m = resolve_method(g, method, S);
  uint32_t path = method_path(m);
  if (reach_dev && path == MSBFS_PATH_CTA) path = MSBFS_PATH_HYBRID;
  CtaShape cta{};
  if (path == MSBFS_PATH_CTA &&
      !cta_launch_shape((uint32_t)g->V, eng->device, true, g->erec != nullptr, S, &cta))
    path = MSBFS_PATH_HYBRID;
  const int cta_grid = std::max(1, (int)((uint64_t)cta.grid * eng->sm_share / 100));
  if (!g->sym && path != MSBFS_PATH_CTA && !g->coff)
    return set_err(eng, MSBFS_ERR_INVALID_GRAPH, "missing transpose");

  eng->last = msbfs_stats{};
  eng->last.method = (uint32_t)m;
  eng->last.path = path;
  eng->last_level_path = path != MSBFS_PATH_CTA;
  if ((rc = grow(eng, &eng->d_sources, &eng->d_sources_cap, S))) return rc;
  CK(cudaEventRecord(eng->ev_start, eng->stream));
  CK(cudaMemcpyAsync(eng->d_sources, sources, S * sizeof(uint32_t), cudaMemcpyHostToDevice,
                     eng->stream));
  const size_t V = g->V;

  if (path == MSBFS_PATH_CTA) {
    // Cluster mode: `blocks` stays a multiple of the cluster size, one
    // queue slab per cluster.
    const int cl = std::max(1, cta.cluster);
    const int blocks = std::max(cl, std::min<int>(cta_grid, (int)std::min<size_t>(S * cl, 1u << 30)) / cl * cl);
    if ((rc = grow(eng, &eng->d_cta_queue, &eng->d_cta_queue_cap, (size_t)(blocks / cl) * V)))
      return rc;
    if (cta.global_bits &&
        (rc = grow(eng, &eng->d_cta_bits, &eng->d_cta_bits_cap, (size_t)blocks * ((V + 31) / 32))))
      return rc;
    CK(cudaMemsetAsync(eng->d_work, 0, sizeof(uint32_t), eng->stream));
    CtaParams cp{};
    cp.V = (uint32_t)V;
    cp.off = g->off;
    cp.idx = g->idx;
    cp.sources = eng->d_sources;
    cp.num_sources = (uint32_t)S;
    cp.dist = dist_dev;
    cp.gqueue = eng->d_cta_queue;
    cp.work = eng->d_work;
    cp.stats = stats_dev;
    cp.gbits = cta.global_bits ? eng->d_cta_bits : nullptr;
    cp.erec = g->erec;
    launch_cta(cp, cta, blocks, eng->stream);
    CK(cudaGetLastError());
    eng->last.passes = 1;
    eng->last.cta_cluster = cta.cluster > 1 ? (uint32_t)cta.cluster : 0u;
    eng->last_passes = 0;
    if (host_out) {
      CK(cudaMemcpyAsync(host_out, dist_dev, S * V * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                         eng->stream));
    }
    CK(cudaEventRecord(eng->ev_stop, eng->stream));
    return MSBFS_OK;
  }

  const uint32_t mode = path == MSBFS_PATH_PUSH   ? MODE_PUSH
                        : path == MSBFS_PATH_PULL ? MODE_PULL
                                                  : MODE_HYBRID;
  const uint32_t W = choose_words(eng, S);
  const size_t PW = (size_t)W * 32;
  const size_t passes = (S + PW - 1) / PW;
  Workspace* w = nullptr;
  if ((rc = get_workspace(eng, g, W, mode, &w))) return rc;
  const bool reduce = stats_dev != nullptr;
  if (reduce && !eng->host_loop && w->exec[0] && !w->exec[1] &&
      build_graph_exec(eng, w, PASS_STATS) != MSBFS_OK) {
    eng->host_loop = true;
    cudaGetLastError();
  }
  // Split materialisation (graph loop only): the pass's graph ends after
  // the byte rows; the u32 rows and the cleanup follow as plain launches
  // while the host widens the bytes.
  bool split = split_frac > 0.0 && dist8_dev && dist_dev && !reduce && !reach_dev &&
               eng->profiling == 0 && !eng->host_loop && w->exec[PASS_ROWS];
  if (split && !w->exec[PASS_BYTES] && build_graph_exec(eng, w, PASS_BYTES) != MSBFS_OK) {
    cudaGetLastError();
    split = false;
  }
  eng->last_split = split;
  eng->split_rows.assign(passes, 0);
  while (split && eng->split_events.size() < passes) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    eng->split_events.push_back(e);
  }
  if (passes > eng->h_ctl_cap) {
    CK(cudaStreamSynchronize(eng->stream));
    if (eng->h_ctl) cudaFreeHost(eng->h_ctl);
    eng->h_ctl = nullptr;
    eng->h_ctl_cap = 0;
    CK(cudaMallocHost((void**)&eng->h_ctl, passes * sizeof(LevelCtl)));
    eng->h_ctl_cap = passes;
  }
  eng->last.passes = (uint32_t)passes;
  eng->last.words_per_vertex = W;
  eng->last_passes = passes;
  if (eng->profiling) {
    if (passes > eng->h_log_passes) {
      CK(cudaStreamSynchronize(eng->stream));
      if (eng->h_log) cudaFreeHost(eng->h_log);
      eng->h_log = nullptr;
      eng->h_log_passes = 0;
      CK(cudaMallocHost((void**)&eng->h_log, passes * LOG_CAP * sizeof(LevelRec)));
      eng->h_log_passes = passes;
    }
    eng->pass_event_ms.assign(passes, {});
  }
  const size_t wpv = (S + 31) / 32;
  // Any early return below leaves passes half-queued: the workspace is
  // retired unless the loop completes.
  w->dirty = true;
  for (size_t ps = 0; ps < passes; ++ps) {
    const size_t s0 = ps * PW;
    const size_t np = std::min(PW, S - s0);
    PassDesc d{};
    d.sources = eng->d_sources + s0;
    d.dist = dist_dev ? dist_dev + s0 * V : nullptr;
    d.reach = reach_dev;
    d.stats = stats_dev ? stats_dev + s0 : nullptr;
    d.dist8 = dist8_dev ? dist8_dev + s0 * V : nullptr;
    d.num_sources = (uint32_t)np;
    d.reach_wpv = (uint32_t)wpv;
    d.reach_col = (uint32_t)(ps * W);
    d.row_split = split ? (uint32_t)(split_frac * (double)np) / 32u * 32u : 0u;
    eng->split_rows[ps] = d.row_split;
    // Pageable source: the copy is staged before the call returns, so the
    // stack descriptor can go out of scope.
    CK(cudaMemcpyAsync(w->d_desc, &d, sizeof d, cudaMemcpyHostToDevice, eng->stream));
    if (eng->profiling >= 2) {
      if ((rc = run_pass_profiled(eng, w, reduce, &eng->pass_event_ms[ps]))) return rc;
    } else if (split) {
      CK(cudaGraphLaunch(w->exec[PASS_BYTES], eng->stream));
      CK(cudaMemcpyAsync(&eng->h_ctl[ps], w->d_ctl, sizeof(LevelCtl), cudaMemcpyDeviceToHost,
                         eng->stream));
      CK(cudaEventRecord(eng->split_events[ps], eng->stream));
      launch_materialize(w->p, w->k, false, eng->stream, MAT_WIDE);
      launch_cleanup(w->p, eng->stream);
      CK(cudaGetLastError());
    } else if (w->exec[reduce] && !eng->host_loop) {
      CK(cudaGraphLaunch(w->exec[reduce], eng->stream));
    } else {
      if ((rc = run_pass_host_loop(eng, w, reduce))) return rc;
    }
    CK(cudaMemcpyAsync(&eng->h_ctl[ps], w->d_ctl, sizeof(LevelCtl), cudaMemcpyDeviceToHost,
                       eng->stream));
    if (eng->profiling)
      CK(cudaMemcpyAsync(eng->h_log + ps * LOG_CAP, w->d_log, LOG_CAP * sizeof(LevelRec),
                         cudaMemcpyDeviceToHost, eng->stream));
    if (host_out) {
      CK(cudaEventRecord(eng->ev_pass, eng->stream));
      CK(cudaStreamWaitEvent(eng->copy_stream, eng->ev_pass, 0));
      CK(cudaMemcpyAsync(host_out + s0 * V, dist_dev + s0 * V, np * V * sizeof(uint32_t),
                         cudaMemcpyDeviceToHost, eng->copy_stream));
    }
  }
  w->dirty = false;
  if (host_reach) {
    CK(cudaMemcpyAsync(host_reach, reach_dev, V * wpv * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost, eng->stream));
  }
  if (host_out) {
    CK(cudaEventRecord(eng->ev_copies, eng->copy_stream));
    CK(cudaStreamWaitEvent(eng->stream, eng->ev_copies, 0));
  }
  CK(cudaEventRecord(eng->ev_stop, eng->stream));
  return MSBFS_OK;
}

int finish_call(msbfs_engine* eng, msbfs_stats* stats) {
  CK(cudaEventSynchronize(eng->ev_stop));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, eng->ev_start, eng->ev_stop);
  eng->last.gpu_ms = ms;
  uint32_t status = 0, check_site = 0;
  for (size_t i = 0; i < eng->last_passes; ++i) {
    const LevelCtl& c = eng->h_ctl[i];
    if (!check_site) check_site = c.check_site;
    eng->last.levels = std::max(eng->last.levels, c.level + 1);
    eng->last.push_levels += c.push_levels;
    eng->last.pull_levels += c.pull_levels;
    eng->last.reached_pairs += c.pairs;
    status |= c.status;
  }
  eng->log.clear();
  if (eng->profiling && eng->h_log) {
    for (size_t ps = 0; ps < eng->last_passes; ++ps) {
      const LevelCtl& c = eng->h_ctl[ps];
      const uint32_t nlev = std::min<uint32_t>(c.level + 1, LOG_CAP);
      const std::vector<float>* ev =
          ps < eng->pass_event_ms.size() ? &eng->pass_event_ms[ps] : nullptr;
      for (uint32_t L = 0; L < nlev; ++L) {
        const LevelRec& r = eng->h_log[ps * LOG_CAP + L];
        msbfs_level_record o{};
        o.pass = (uint32_t)ps;
        o.level = r.level;
        o.dir = r.dir;
        o.frontier_vertices = r.frontier_vertices;
        o.frontier_entries = r.frontier_entries;
        o.active = r.active;
        o.edges = r.edges;
        o.new_vertices = r.new_vertices;
        o.new_pairs = r.new_pairs;
        o.rows = r.rows;
        o.device_ms = r.t_end > r.t_start ? (double)(r.t_end - r.t_start) * 1e-6 : 0.0;
        o.event_ms = (ev && L < ev->size() && !ev->empty()) ? (*ev)[L] : 0.0;
        eng->log.push_back(o);
      }
      if (ev && !ev->empty()) {
        msbfs_level_record m{};
        m.pass = (uint32_t)ps;
        m.level = c.level;
        m.dir = MSBFS_DIR_MATERIALIZE;
        m.event_ms = ev->back();
        eng->log.push_back(m);
      }
    }
  }
  if (stats) *stats = eng->last;
  if (status & STATUS_CHECK)
    return set_err(eng, MSBFS_ERR_CUDA,
                   "bounds check failed at site " + std::to_string(check_site));
  if (status & STATUS_LEVEL_CAP) return set_err(eng, MSBFS_ERR_TIMEOUT, "level cap reached");
  if (status & STATUS_BAD_SOURCE) return set_err(eng, MSBFS_ERR_SOURCE_OOB, "source out of range");
  return MSBFS_OK;
}

// Slice table of in-edge lists longer than `split` and the bottom-up work
// list of the other vertices with in-edges, from the graph's host CSC
// offsets. Rebuilt when the autotuner changes the slice length; the caller
// drops the workspaces that point at the old tables first.
int build_bottom_up_tables(msbfs_engine* eng, msbfs_graph* g, uint32_t split) {
  const size_t V = g->V;
  const std::vector<uint32_t>& coff = g->h_coff;
  cudaFree(g->hchunks);
  cudaFree(g->order);
  g->hchunks = nullptr;
  g->order = nullptr;
  g->split = split;
  g->n_heavy = 0;
  std::vector<HeavyChunk> chunks;
  for (size_t v = 0; v < V; ++v) {
    const uint32_t indeg = coff[v + 1] - coff[v];
    if (indeg <= split) continue;
    const uint32_t nch = (indeg + split - 1) / split;
    for (uint32_t j = 0; j < nch; ++j) chunks.push_back(HeavyChunk{(uint32_t)v, j, nch, g->n_heavy});
    g->n_heavy++;
  }
  // Longest lists first so their slices start early in every bottom-up step.
  std::stable_sort(chunks.begin(), chunks.end(), [](const HeavyChunk& a, const HeavyChunk& b) {
    return a.nch > b.nch;
  });
  g->n_hchunks = (uint32_t)chunks.size();
  CK(cudaMalloc((void**)&g->hchunks, std::max<size_t>(chunks.size(), 1) * sizeof(HeavyChunk)));
  if (!chunks.empty())
    CK(cudaMemcpy(g->hchunks, chunks.data(), chunks.size() * sizeof(HeavyChunk),
                  cudaMemcpyHostToDevice));
  // Bottom-up work list: the vertices with 0 < in-degree <= split, ascending
  // ids (neighbouring vertices share cache lines of the visited and frontier
  // rows). MSBFS_ORDER_WINDOW > 1 sorts by in-degree, descending, within
  // windows of that many entries, so the groups of a warp scan in-edge lists
  // of similar length; on R-MAT scale 22, S=512 the lost locality outweighs
  // the balance (window 256: +8%, window 1024: +10% bottom-up time), so the
  // default keeps plain id order.
#ifndef MSBFS_ORDER_WINDOW
#define MSBFS_ORDER_WINDOW 0
#endif
  std::vector<uint32_t> order;
  order.reserve(V);
  for (size_t v = 0; v < V; ++v) {
    const uint32_t d = coff[v + 1] - coff[v];
    if (d > 0 && d <= split) order.push_back((uint32_t)v);
  }
  const size_t win = MSBFS_ORDER_WINDOW;
  if (win > 1) {
    auto deg_desc = [&](uint32_t a, uint32_t b) {
      return coff[a + 1] - coff[a] > coff[b + 1] - coff[b];
    };
    for (size_t i = 0; i < order.size(); i += win)
      std::stable_sort(order.begin() + i, order.begin() + std::min(order.size(), i + win),
                       deg_desc);
  }
  g->n_order = (uint32_t)order.size();
  // Each entry carries the vertex and its in-edge range, so a bottom-up
  // step starts a vertex's scan one dependent load earlier.
  std::vector<uint4> ent(order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    const uint32_t v = order[i];
    ent[i] = make_uint4(v, coff[v], coff[v + 1], 0u);
  }
  CK(cudaMalloc((void**)&g->order, std::max<size_t>(ent.size(), 1) * sizeof(uint4)));
  if (!ent.empty())
    CK(cudaMemcpy(g->order, ent.data(), ent.size() * sizeof(uint4), cudaMemcpyHostToDevice));
  return MSBFS_OK;
}

int upload_graph(msbfs_engine* eng, size_t V, size_t E, const uint32_t* off, const uint32_t* idx,
                 msbfs_graph** out) {
  if (!eng || !out) return MSBFS_ERR_INVALID_ARGUMENT;
  if (V >= 0xFFFFFFFFull || E > 0xFFFFFFFFull)
    return set_err(eng, MSBFS_ERR_INVALID_GRAPH, "graph exceeds u32 indices");
  std::string why = msbfs::validate(V, E, off, idx, E);
  if (!why.empty()) return set_err(eng, MSBFS_ERR_INVALID_GRAPH, why);
  auto g = std::make_unique<msbfs_graph>();
  g->eng = eng;
  static std::atomic<uint64_t> next_graph_id{1};
  g->id = next_graph_id++;
  g->V = V;
  g->E = E;
  g->max_deg = msbfs::max_degree(V, off);
  msbfs::HostCsr t = msbfs::transpose(V, E, off, idx);
  g->sym = std::equal(t.off.begin(), t.off.end(), off) &&
           (E == 0 || std::memcmp(t.idx.data(), idx, E * 4) == 0);
  CK(cudaSetDevice(eng->device));
  CK(cudaMalloc((void**)&g->off, (V + 1) * 4));
  CK(cudaMalloc((void**)&g->idx, std::max<size_t>(E, 1) * 4));
  CK(cudaMemcpy(g->off, off, (V + 1) * 4, cudaMemcpyHostToDevice));
  if (E) CK(cudaMemcpy(g->idx, idx, E * 4, cudaMemcpyHostToDevice));
  if (g->sym) {
    g->coff = g->off;
    g->cidx = g->idx;
  } else {
    CK(cudaMalloc((void**)&g->coff, (V + 1) * 4));
    CK(cudaMalloc((void**)&g->cidx, std::max<size_t>(E, 1) * 4));
    CK(cudaMemcpy(g->coff, t.off.data(), (V + 1) * 4, cudaMemcpyHostToDevice));
    if (E) CK(cudaMemcpy(g->cidx, t.idx.data(), E * 4, cudaMemcpyHostToDevice));
  }
  g->h_coff = std::move(t.off);
  int rc = build_bottom_up_tables(eng, g.get(), eng->split);
  if (rc) return rc;
  // Road-like graphs (the ones the router sends to the CTA path) get edge
  // records, 16 bytes per edge, so a CTA-path level costs one dependent L2
  // round trip instead of three.
  if (is_road_like(g.get()) && E > 0) {
    CK(cudaMalloc((void**)&g->erec, E * sizeof(uint4)));
    launch_edge_records((uint32_t)V, g->off, g->idx, g->erec, eng->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(eng->stream));
  }
  *out = g.release();
  return MSBFS_OK;
}

void free_graph(msbfs_graph* g) {
  if (!g) return;
  std::vector<msbfs_engine*> engines = g->users;
  engines.push_back(g->eng);
  for (msbfs_engine* eng : engines) {
    if (!eng) continue;
    std::lock_guard<std::mutex> lk(eng->mu);
    cudaSetDevice(eng->device);
    cudaStreamSynchronize(eng->stream);
    for (auto it = eng->ws.begin(); it != eng->ws.end();)
      if (std::get<0>(it->first) == g->id)
        it = eng->ws.erase(it);
      else
        ++it;
  }
  if (!g->sym) {
    cudaFree(g->coff);
    cudaFree(g->cidx);
  }
  cudaFree(g->off);
  cudaFree(g->idx);
  cudaFree(g->hchunks);
  cudaFree(g->order);
  cudaFree(g->erec);
  delete g;
}

// Copies n byte distances from the device to the host through a ring of
// page-locked chunk slots (one event per slot on the copy stream) while
// every hardware thread widens each chunk, once it has landed, into u32
// (0xFF -> 0xFFFFFFFF) at `out`: the host link carries a quarter of the
// bytes, and the host's cores, which write memory faster than the link
// delivers it, do the widening. The calling thread issues the copies; a
// slot is refilled only after all workers have widened its previous chunk,
// and a worker waits for its chunk's copy to be issued before it waits on
// the slot's event.
int widen_to_host(msbfs_engine* eng, const uint8_t* src, uint32_t* out, size_t n) {
  if (n == 0) return MSBFS_OK;
  constexpr size_t CHUNK = 32u << 20, SLOTS = 16;
  const size_t stage = std::min(n, CHUNK * SLOTS);
  if (stage > eng->h_dist8_cap) {
    if (eng->h_dist8) cudaFreeHost(eng->h_dist8);
    eng->h_dist8 = nullptr;
    eng->h_dist8_cap = 0;
    CK(cudaHostAlloc((void**)&eng->h_dist8, stage, cudaHostAllocDefault));
    eng->h_dist8_cap = stage;
  }
  while (eng->chunk_events.size() < SLOTS) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    eng->chunk_events.push_back(e);
  }
  const size_t nchunks = (n + CHUNK - 1) / CHUNK;
  const unsigned T = std::max(1u, std::thread::hardware_concurrency());
  std::mutex mu;
  std::condition_variable cv;
  size_t issued = 0, widened = 0;  // chunks issued / widened by every worker (in order)
  unsigned slot_done[SLOTS] = {};
  bool failed = false;
  const uint8_t* ring = eng->h_dist8;
  std::vector<std::thread> workers;
  for (unsigned k = 0; k < T; ++k) {
    workers.emplace_back([&, k] {
      cudaSetDevice(eng->device);
      for (size_t c = 0; c < nchunks; ++c) {
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return issued > c || failed; });
          if (failed) return;
        }
        const size_t slot = c % SLOTS;
        if (cudaEventSynchronize(eng->chunk_events[slot]) != cudaSuccess) {
          std::lock_guard<std::mutex> lk(mu);
          failed = true;
          cv.notify_all();
          return;
        }
        const size_t b = c * CHUNK, len = std::min(CHUNK, n - b);
        const size_t lo = len * k / T, hi = len * (k + 1) / T;
        const uint8_t* in = ring + slot * CHUNK;
        uint32_t* o = out + b;
        for (size_t i = lo; i < hi; ++i) {
          const uint32_t d = in[i];
          o[i] = d == 0xFFu ? 0xFFFFFFFFu : d;
        }
        std::lock_guard<std::mutex> lk(mu);
        if (++slot_done[slot] == T) {
          slot_done[slot] = 0;
          ++widened;
          cv.notify_all();
        }
      }
    });
  }
  cudaError_t err = cudaSuccess;
  for (size_t c = 0; c < nchunks && err == cudaSuccess; ++c) {
    const size_t slot = c % SLOTS, b = c * CHUNK, len = std::min(CHUNK, n - b);
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return c < SLOTS || widened + SLOTS > c || failed; });
      if (failed) break;
    }
    err = cudaMemcpyAsync(eng->h_dist8 + slot * CHUNK, src + b, len, cudaMemcpyDeviceToHost,
                          eng->copy_stream);
    if (err == cudaSuccess) err = cudaEventRecord(eng->chunk_events[slot], eng->copy_stream);
    std::lock_guard<std::mutex> lk(mu);
    if (err == cudaSuccess)
      issued = c + 1;
    else
      failed = true;
    cv.notify_all();
  }
  for (std::thread& t : workers) t.join();
  if (failed || err != cudaSuccess) {
    cudaGetLastError();
    return set_err(eng, MSBFS_ERR_CUDA, "byte-row copy failed");
  }
  return MSBFS_OK;
}

// Blocking run into caller-owned host memory.
int run_host(msbfs_engine* eng, int method, const msbfs_graph* g, const uint32_t* sources,
             size_t S, uint32_t* out, msbfs_stats* stats) {
  int rc = validate_call(eng, g, sources, S);
  if (rc) return rc;
  if (stats) *stats = msbfs_stats{};
  if (S == 0) return MSBFS_OK;
  if (!out) return set_err(eng, MSBFS_ERR_INVALID_ARGUMENT, "out is null");
  CK(cudaSetDevice(eng->device));
  // Page-locked host output (cudaHostAlloc / cudaHostRegister) is written by
  // the materialise kernel directly over the host link, in 512-byte row
  // segments, instead of being staged in HBM and copied afterwards. The
  // CTA-per-source path stores 4-byte distances as it discovers them, which
  // the host link serves ~9x slower than a staged copy, so it keeps staging.
  const bool cta = method_path(resolve_method(g, method, S)) == MSBFS_PATH_CTA;
  const size_t V = g->V;
  uint32_t* zc = nullptr;  // device address of page-locked `out`
  if (eng->zero_copy && !cta) {
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, out) == cudaSuccess &&
        attr.type == cudaMemoryTypeHost && attr.devicePointer)
      zc = (uint32_t*)attr.devicePointer;
    else
      cudaGetLastError();
  }
  // Byte rows (decided on the device for each pass: all its distances fit a
  // byte) widened by the host's cores. Pageable output: a byte pass's rows
  // all travel as bytes; a deeper pass writes u32 rows to HBM staging,
  // copied afterwards. Page-locked output: the link alone is about as fast
  // as link + widening, which share the host's memory bandwidth, so a pass
  // splits its rows -- the first split_frac written as u32 straight over the
  // link while the host widens the rest, which travel as bytes. Without room
  // for the byte rows the call keeps u32 rows throughout.
  const bool use_bytes = eng->narrow && !cta && (!zc || eng->split_frac < 1.0);
  if (use_bytes && grow(eng, &eng->d_dist8, &eng->d_dist8_cap, S * V) == MSBFS_OK) {
    uint32_t* wide = zc;
    if (!wide) {
      if ((rc = grow(eng, &eng->d_dist, &eng->d_dist_cap, S * V))) return rc;
      wide = eng->d_dist;
    }
    if ((rc = enqueue_call(eng, method, g, sources, S, wide, nullptr, nullptr, nullptr, nullptr,
                           eng->d_dist8, zc ? eng->split_frac : 0.0)))
      return rc;
    const size_t PW = (size_t)eng->last.words_per_vertex * 32;
    if (eng->last_split) {
      // Each pass's bytes are widened as soon as they exist, while the GPU
      // writes its u32 rows and runs later passes.
      for (size_t ps = 0; ps < eng->last_passes; ++ps) {
        CK(cudaEventSynchronize(eng->split_events[ps]));
        if (!eng->h_ctl[ps].narrow) continue;
        const size_t s0 = ps * PW, np = std::min(PW, S - s0), r0 = eng->split_rows[ps];
        if ((rc = widen_to_host(eng, eng->d_dist8 + (s0 + r0) * V, out + (s0 + r0) * V,
                                (np - r0) * V)))
          return rc;
      }
      return finish_call(eng, stats);
    }
    if ((rc = finish_call(eng, stats))) return rc;
    for (size_t ps = 0; ps < eng->last_passes; ++ps) {
      const size_t s0 = ps * PW, np = std::min(PW, S - s0);
      if (eng->h_ctl[ps].narrow) {
        if ((rc = widen_to_host(eng, eng->d_dist8 + s0 * V, out + s0 * V, np * V))) return rc;
      } else if (!zc) {
        CK(cudaMemcpy(out + s0 * V, eng->d_dist + s0 * V, np * V * sizeof(uint32_t),
                      cudaMemcpyDeviceToHost));
      }
    }
    return MSBFS_OK;
  }
  if (zc) {
    if ((rc = enqueue_call(eng, method, g, sources, S, zc, nullptr, nullptr, nullptr)))
      return rc;
    return finish_call(eng, stats);
  }
  const size_t total = S * V;
  if ((rc = grow(eng, &eng->d_dist, &eng->d_dist_cap, total))) return rc;
  if ((rc = enqueue_call(eng, method, g, sources, S, eng->d_dist, nullptr, out, nullptr)))
    return rc;
  return finish_call(eng, stats);
}

}  // namespace

// ===================================================================== C ABI

extern "C" {

int msbfs_engine_create(int device, int method, msbfs_engine** out) {
  if (!out) return MSBFS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (method < 0 || method > MSBFS_METHOD_AUTO) return MSBFS_ERR_INVALID_ARGUMENT;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return MSBFS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return MSBFS_ERR_NO_DEVICE;
  auto eng = std::make_unique<msbfs_engine>();
  eng->device = device;
  eng->method = method;
  msbfs_engine* e = eng.get();
  if (cudaSetDevice(device) != cudaSuccess) return MSBFS_ERR_CUDA;
  cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev_start) != cudaSuccess || cudaEventCreate(&e->ev_stop) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_pass, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_copies, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc((void**)&e->d_work, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc((void**)&e->d_counter, sizeof(unsigned long long)) != cudaSuccess)
    return MSBFS_ERR_CUDA;
  e->stream = e->own_stream;
  const char* hl = getenv("MSBFS_HOST_LOOP");
  e->host_loop = hl && hl[0] == '1';
  const char* zc = getenv("MSBFS_ZERO_COPY");
  e->zero_copy = !(zc && zc[0] == '0');
  const char* nr = getenv("MSBFS_NARROW");
  e->narrow = !(nr && nr[0] == '0');
  const char* mw = getenv("MSBFS_MAT_WAVES");
  if (mw) e->mat_waves = (uint32_t)std::max(0, atoi(mw));
  const char* sr = getenv("MSBFS_SPLIT_ROWS");
  if (sr) e->split_frac = std::min(1.0, std::max(0.0, atof(sr)));
  *out = eng.release();
  return MSBFS_OK;
}

void msbfs_engine_destroy(msbfs_engine* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  cudaStreamSynchronize(e->copy_stream);
  e->ws.clear();
  cudaFree(e->d_sources);
  cudaFree(e->d_dist);
  cudaFree(e->d_dist8);
  if (e->h_dist8) cudaFreeHost(e->h_dist8);
  for (cudaEvent_t ev : e->chunk_events) cudaEventDestroy(ev);
  for (cudaEvent_t ev : e->split_events) cudaEventDestroy(ev);
  cudaFree(e->d_reach);
  cudaFree(e->d_cta_queue);
  cudaFree(e->d_cta_bits);
  cudaFree(e->d_work);
  cudaFree(e->d_counter);
  cudaFree(e->d_sstats);
  if (e->h_ctl) cudaFreeHost(e->h_ctl);
  if (e->h_log) cudaFreeHost(e->h_log);
  for (cudaEvent_t ev : e->lvl_events) cudaEventDestroy(ev);
  cudaEventDestroy(e->ev_start);
  cudaEventDestroy(e->ev_stop);
  cudaEventDestroy(e->ev_pass);
  cudaEventDestroy(e->ev_copies);
  cudaStreamDestroy(e->own_stream);
  cudaStreamDestroy(e->copy_stream);
  delete e;
}

int msbfs_engine_method(const msbfs_engine* e) { return e ? e->method : -1; }

const char* msbfs_engine_last_error(const msbfs_engine* e) {
  return e ? e->last_error.c_str() : "null engine";
}

int msbfs_engine_set_stream(msbfs_engine* e, void* s) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  e->stream = s ? (cudaStream_t)s : e->own_stream;
  return MSBFS_OK;
}

int msbfs_engine_set_tuning(msbfs_engine* e, uint32_t max_words, uint32_t alpha, uint32_t beta) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  if (max_words) {
    if (max_words > 64 || (max_words & (max_words - 1)))
      return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "max_words_per_pass must be a power of two <= 64");
    e->max_words = max_words;
  }
  if (alpha) e->alpha = alpha;
  if (beta) e->beta = beta;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  e->ws.clear();  // thresholds are baked into the captured graphs
  return MSBFS_OK;
}

int msbfs_engine_set_sm_share(msbfs_engine* e, uint32_t percent) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  if (percent < 1 || percent > 100)
    return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "sm share must be 1..100 percent");
  std::lock_guard<std::mutex> lk(e->mu);
  e->sm_share = percent;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  e->ws.clear();  // grid sizes are baked into the captured graphs
  return MSBFS_OK;
}

int msbfs_engine_set_level_cap(msbfs_engine* e, uint32_t max_levels) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  e->level_cap = max_levels;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  e->ws.clear();  // the cap is baked into the captured graphs
  return MSBFS_OK;
}

int msbfs_engine_set_profiling(msbfs_engine* e, int level) {
  if (!e || level < 0 || level > 3) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  auto counting = [](int l) { return l == 1 || l == 2; };
  if (counting(e->profiling) != counting(level)) {
    // The captured graphs hold the counting or the production level kernels.
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    e->ws.clear();
  }
  e->profiling = level;
  return MSBFS_OK;
}

int msbfs_engine_level_log(const msbfs_engine* e, msbfs_level_record* out, size_t cap,
                           size_t* count) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  const size_t n = e->log.size();
  if (count) *count = n;
  if (out) std::memcpy(out, e->log.data(), std::min(cap, n) * sizeof(msbfs_level_record));
  return MSBFS_OK;
}

int msbfs_select_auto_method(size_t V, size_t E, const uint32_t* off, size_t S) {
  msbfs_graph g;
  g.V = V;
  g.E = E;
  g.max_deg = (V && off) ? msbfs::max_degree(V, off) : 0;
  return resolve_method(&g, MSBFS_METHOD_AUTO, S);
}

int msbfs_graph_create(msbfs_engine* e, size_t V, size_t E, const uint32_t* off,
                       const uint32_t* idx, msbfs_graph** out) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  return upload_graph(e, V, E, off, idx, out);
}

void msbfs_graph_destroy(msbfs_graph* g) { free_graph(g); }

}  // extern "C"

// Lets another engine of the same device run on `g` without a second upload
// (the served form's slots share one resident graph). Not part of the C ABI:
// destroying `g` drops the workspaces of every engine attached to it, so `g`
// must be destroyed before any of them.
int msbfs_graph_attach(msbfs_graph* g, msbfs_engine* e) {
  if (!g || !e || !g->eng) return MSBFS_ERR_INVALID_ARGUMENT;
  if (e->device != g->eng->device)
    return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "graph lives on another device");
  if (e != g->eng && std::find(g->users.begin(), g->users.end(), e) == g->users.end())
    g->users.push_back(e);
  return MSBFS_OK;
}

extern "C" {

int msbfs_graph_info(const msbfs_graph* g, size_t* V, size_t* E, uint32_t* max_deg, int* sym) {
  if (!g) return MSBFS_ERR_INVALID_ARGUMENT;
  if (V) *V = g->V;
  if (E) *E = g->E;
  if (max_deg) *max_deg = g->max_deg;
  if (sym) *sym = g->sym ? 1 : 0;
  return MSBFS_OK;
}

int msbfs_run_ms_bfs(msbfs_engine* e, const msbfs_graph* g, const uint32_t* sources, size_t S,
                     uint32_t* out, msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  return run_host(e, e->method, g, sources, S, out, stats);
}

int msbfs_run_ms_bfs_with_method(msbfs_engine* e, int method, const msbfs_graph* g,
                                 const uint32_t* sources, size_t S, uint32_t* out,
                                 msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  if (method < 0 || method > MSBFS_METHOD_AUTO)
    return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "unknown method");
  std::lock_guard<std::mutex> lk(e->mu);
  return run_host(e, method, g, sources, S, out, stats);
}

int msbfs_run_ms_bfs_csr(msbfs_engine* e, size_t V, size_t E, const uint32_t* off,
                         const uint32_t* idx, const uint32_t* sources, size_t S, uint32_t* out,
                         msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  if (S == 0) {
    if (stats) *stats = msbfs_stats{};
    return MSBFS_OK;
  }
  msbfs_graph* g = nullptr;
  int rc;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    rc = upload_graph(e, V, E, off, idx, &g);
    if (rc == MSBFS_OK) rc = run_host(e, e->method, g, sources, S, out, stats);
  }
  free_graph(g);
  return rc;
}

int msbfs_run_ms_bfs_device(msbfs_engine* e, int method, const msbfs_graph* g,
                            const uint32_t* sources, size_t S, uint32_t* out_device) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  if (method < 0 || method > MSBFS_METHOD_AUTO)
    return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "unknown method");
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  int rc = validate_call(e, g, sources, S);
  if (rc) return rc;
  e->last = msbfs_stats{};
  e->last_passes = 0;
  if (S == 0) {
    CK(cudaEventRecord(e->ev_start, e->stream));
    CK(cudaEventRecord(e->ev_stop, e->stream));
    return MSBFS_OK;
  }
  if (!out_device) return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "out is null");
  CK(cudaSetDevice(e->device));
  return enqueue_call(e, method, g, sources, S, out_device, nullptr, nullptr, nullptr);
}

static_assert(sizeof(SourceStats) == sizeof(msbfs_source_stats), "stats layout");

int msbfs_run_ms_bfs_stats_device(msbfs_engine* e, int method, const msbfs_graph* g,
                                  const uint32_t* sources, size_t S,
                                  msbfs_source_stats* stats_device) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  if (method < 0 || method > MSBFS_METHOD_AUTO)
    return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "unknown method");
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  int rc = validate_call(e, g, sources, S);
  if (rc) return rc;
  e->last = msbfs_stats{};
  e->last_passes = 0;
  if (S == 0) {
    CK(cudaEventRecord(e->ev_start, e->stream));
    CK(cudaEventRecord(e->ev_stop, e->stream));
    return MSBFS_OK;
  }
  if (!stats_device) return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "stats is null");
  CK(cudaSetDevice(e->device));
  return enqueue_call(e, method, g, sources, S, nullptr, nullptr, nullptr, nullptr,
                      reinterpret_cast<SourceStats*>(stats_device));
}

int msbfs_run_ms_bfs_stats(msbfs_engine* e, const msbfs_graph* g, const uint32_t* sources,
                           size_t S, msbfs_source_stats* out, msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  int rc = validate_call(e, g, sources, S);
  if (rc) return rc;
  if (stats) *stats = msbfs_stats{};
  if (S == 0) return MSBFS_OK;
  if (!out) return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "out is null");
  CK(cudaSetDevice(e->device));
  if ((rc = grow(e, &e->d_sstats, &e->d_sstats_cap, S))) return rc;
  if ((rc = enqueue_call(e, e->method, g, sources, S, nullptr, nullptr, nullptr, nullptr,
                         e->d_sstats)))
    return rc;
  CK(cudaMemcpyAsync(out, e->d_sstats, S * sizeof(SourceStats), cudaMemcpyDeviceToHost,
                     e->stream));
  CK(cudaEventRecord(e->ev_stop, e->stream));
  return finish_call(e, stats);
}

int msbfs_engine_synchronize(msbfs_engine* e, msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  return finish_call(e, stats);
}

int msbfs_run_reachability(msbfs_engine* e, const msbfs_graph* g, const uint32_t* sources,
                           size_t S, uint32_t* words, msbfs_stats* stats) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  int rc = validate_call(e, g, sources, S);
  if (rc) return rc;
  if (stats) *stats = msbfs_stats{};
  if (S == 0 || g->V == 0) return MSBFS_OK;
  if (!words) return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "words is null");
  CK(cudaSetDevice(e->device));
  const size_t wpv = (S + 31) / 32;
  if ((rc = grow(e, &e->d_reach, &e->d_reach_cap, g->V * wpv))) return rc;
  int method = e->method;
  if (resolve_method(g, method, S) == MSBFS_METHOD_WORKGROUP_PERSISTENT_BFS)
    method = MSBFS_METHOD_PUSH_PULL_ADAPTIVE;
  if ((rc = enqueue_call(e, method, g, sources, S, nullptr, e->d_reach, nullptr, words)))
    return rc;
  return finish_call(e, stats);
}

int msbfs_traversed_edges_device(msbfs_engine* e, const msbfs_graph* g, const uint32_t* dist,
                                 size_t S, uint64_t* out_edges) {
  if (!e || !g || !out_edges) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  *out_edges = 0;
  if (S == 0 || g->V == 0) return MSBFS_OK;
  CK(cudaSetDevice(e->device));
  launch_traversed_edges((uint32_t)g->V, g->off, dist, (uint32_t)S, e->d_counter, e->stream);
  CK(cudaGetLastError());
  unsigned long long h = 0;
  CK(cudaMemcpyAsync(&h, e->d_counter, sizeof h, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  *out_edges = h;
  return MSBFS_OK;
}

}  // extern "C"

// ============================================================ level autotuner

namespace {

// Settings of the level-synchronous path that the autotuner varies.
struct LevelSettings {
  uint32_t words, alpha, beta, split, bits_div, heavy;
  uint32_t& at(int i) {
    return i == 0 ? words : i == 1 ? alpha : i == 2 ? beta : i == 3 ? split : i == 4 ? bits_div
                                                                                  : heavy;
  }
  bool operator==(const LevelSettings& o) const {
    return words == o.words && alpha == o.alpha && beta == o.beta && split == o.split &&
           bits_div == o.bits_div && heavy == o.heavy;
  }
};

// The thresholds are baked into an engine's captured graphs, so its
// workspaces are dropped; a new slice length rebuilds the graph's bottom-up
// tables (done only when no other engine runs on the graph).
int apply_settings(msbfs_engine* eng, msbfs_graph* g, const LevelSettings& s) {
  CK(cudaStreamSynchronize(eng->stream));
  CK(cudaStreamSynchronize(eng->copy_stream));
  eng->ws.clear();
  eng->max_words = s.words;
  eng->alpha = s.alpha;
  eng->beta = s.beta;
  eng->bits_div = s.bits_div;
  eng->heavy = s.heavy;
  if (s.split != g->split) return build_bottom_up_tables(eng, g, s.split);
  return MSBFS_OK;
}

// Device time (CUDA events) of one per-source-statistics call: the smaller
// of two after a call that builds the workspace.
int time_stats_call(msbfs_engine* eng, msbfs_graph* g, const uint32_t* src, size_t S, int method,
                    double* ms) {
  int rc;
  if ((rc = grow(eng, &eng->d_sstats, &eng->d_sstats_cap, S))) return rc;
  double best = 1e30;
  for (int k = 0; k < 3; ++k) {
    if ((rc = enqueue_call(eng, method, g, src, S, nullptr, nullptr, nullptr, nullptr,
                           eng->d_sstats)))
      return rc;
    msbfs_stats st{};
    if ((rc = finish_call(eng, &st))) return rc;
    if (k > 0) best = std::min(best, st.gpu_ms);
  }
  *ms = best;
  return MSBFS_OK;
}

}  // namespace

extern "C" int msbfs_engine_autotune(msbfs_engine* e, msbfs_graph* g, const uint32_t* sources,
                                     size_t S, const char* cache_path, msbfs_tuning* out) {
  if (!e) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(e->mu);
  msbfs_engine* eng = e;
  int rc = validate_call(e, g, sources, S);
  if (rc) return rc;
  if (S == 0 || g->V == 0) return set_err(e, MSBFS_ERR_INVALID_ARGUMENT, "autotune needs sources");
  CK(cudaSetDevice(e->device));
  size_t bucket = 1;
  while (bucket < S) bucket <<= 1;
  const std::string key =
      msbfs::graph_class(g->V, g->E, g->max_deg) + "/s" + std::to_string(bucket);
  msbfs_tuning t{};
  std::strncpy(t.class_name, key.c_str(), sizeof t.class_name - 1);
  LevelSettings best{e->max_words, e->alpha, e->beta, g->split, e->bits_div, e->heavy};
  auto report = [&](const LevelSettings& s) {
    // The words a pass of this call uses (a cap above the sources' need
    // makes no difference).
    uint32_t need = 1;
    while (need < (S + 31) / 32 && need < 64) need <<= 1;
    t.max_words_per_pass = std::min(s.words, need);
    t.alpha = s.alpha;
    t.beta = s.beta;
    t.hub_split = s.split;
    t.bitmap_div = s.bits_div;
    t.warp_scan_degree = s.heavy;
    if (out) *out = t;
    return MSBFS_OK;
  };
  const int method = resolve_method(g, e->method, S);
  if (method_path(method) == MSBFS_PATH_CTA) return report(best);
  t.level_path = 1;
  const bool shared = !g->users.empty() || g->eng != e;  // other engines hold its tables
  // Cache: one line per class,
  // "class words alpha beta split bitmap_div warp_scan_degree ms".
  if (cache_path) {
    std::ifstream in(cache_path);
    std::string k;
    LevelSettings s{};
    double ms = 0;
    while (in >> k >> s.words >> s.alpha >> s.beta >> s.split >> s.bits_div >> s.heavy >> ms) {
      if (k != key) continue;
      if (shared) s.split = g->split;
      if ((rc = apply_settings(e, g, s))) return rc;
      t.from_cache = 1;
      t.ms = ms;
      return report(s);
    }
  }
  double best_ms = 0;
  if ((rc = time_stats_call(e, g, sources, S, method, &best_ms))) return rc;
  t.default_ms = best_ms;
  t.trials = 1;
  uint32_t wmax = 1;
  while (wmax < (S + 31) / 32 && wmax < 64) wmax <<= 1;
  const std::vector<std::vector<uint32_t>> cands = {
      {std::max(1u, wmax / 4), std::max(1u, wmax / 2), wmax},  // words per vertex
      {4, 8, 14, 28, 56},                                      // alpha
      {6, 12, 24, 64, 256},                                    // beta
      {256, 512, 1024},                                        // slice length
      {16, 64, 256},                                           // bitmap divisor
      {8, 16, 32, 64}};                                        // warp-scan in-degree
  // One setting at a time, each from the best found so far; a change is
  // kept only when it is at least 2% faster (timing noise).
  for (int i = 0; i < 6; ++i) {
    if (i == 3 && shared) continue;
    const LevelSettings base = best;
    for (uint32_t c : cands[i]) {
      LevelSettings s = base;
      s.at(i) = c;
      if (s == base) continue;
      if ((rc = apply_settings(e, g, s))) return rc;
      double ms = 0;
      if ((rc = time_stats_call(e, g, sources, S, method, &ms))) return rc;
      ++t.trials;
      if (ms < best_ms * 0.98) {
        best_ms = ms;
        best = s;
      }
    }
  }
  if ((rc = apply_settings(e, g, best))) return rc;
  t.ms = best_ms;
  if (cache_path) {
    std::ofstream o(cache_path, std::ios::app);
    o << key << ' ' << best.words << ' ' << best.alpha << ' ' << best.beta << ' ' << best.split
      << ' ' << best.bits_div << ' ' << best.heavy << ' ' << best_ms << '\n';
  }
  return report(best);
}
