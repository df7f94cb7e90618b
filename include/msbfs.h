/*
 * msbfs.h -- C ABI of the GB300 multi-source BFS engine (libmsbfs.so).
 *
 * This is the drop-in boundary for the reference's GPU multi-source BFS path
 * (crates/gpu_bfs, likr-sandbox/webgpu-bfs). Every entry point below names
 * the reference interface it replaces (file:line inside that project). The
 * signatures carry plain pointers and sizes only: no CUDA, PyTorch or C++
 * types cross the boundary, so a Rust `extern "C"` block, ctypes or any other
 * FFI can bind it.
 *
 * Result contract (crates/core/src/lib.rs:21-39): distances are u32 hop
 * counts laid out source-major, dist[s * V + v]; dist[s * V + sources[s]] = 0;
 * unreachable = 0xFFFFFFFF. Duplicate sources are allowed and each gets its
 * own row. Every correct BFS produces identical bytes, so every method below
 * returns the same output for the same graph and sources.
 *
 * Threading: an engine serialises its own calls with an internal mutex (the
 * reference locks one Mutex per pooled method, crates/gpu_bfs/src/engine.rs:
 * 259-281). Distinct engines may be used from distinct threads.
 */
#ifndef MSBFS_H
#define MSBFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSBFS_ABI_VERSION 1

/* ---- status codes (the reference returns anyhow::Error strings) ---------- */
#define MSBFS_OK 0
/* "Source vertex {} at index {} exceeds graph vertex count {}"
 * (crates/gpu_bfs/src/engine.rs:240-248). */
#define MSBFS_ERR_SOURCE_OOB 1
/* V == 0 with S > 0 (engine.rs:233-238). */
#define MSBFS_ERR_EMPTY_GRAPH 2
#define MSBFS_ERR_OOM 3
/* A bounded device-side loop ran out of iterations (reported, never hung). */
#define MSBFS_ERR_TIMEOUT 4
#define MSBFS_ERR_CUDA 5
/* CsrGraph::validate failed (crates/core/src/graph.rs:226-280). */
#define MSBFS_ERR_INVALID_GRAPH 6
#define MSBFS_ERR_INVALID_ARGUMENT 7
#define MSBFS_ERR_NO_DEVICE 8
/* The graph does not fit the fixed scratch of msbfs_run_cta_noalloc. */
#define MSBFS_ERR_SCRATCH_TOO_SMALL 9
/* A Matrix Market file was rejected (details in msbfs_mtx_error). */
#define MSBFS_ERR_PARSE 10

/* ---- methods: same names and order as GpuBfsMethod (engine.rs:33-53) ------
 * Every method produces identical bytes. On GB300 they map onto four kernel
 * paths: level-synchronous bit-parallel push, pull or device-switched hybrid,
 * and the CTA-per-source persistent BFS. */
typedef enum msbfs_method {
  MSBFS_METHOD_NAIVE_SEQUENTIAL = 0,
  MSBFS_METHOD_BATCHED_DENSE_SPMM = 1,
  MSBFS_METHOD_BIT_PARALLEL_32 = 2,
  MSBFS_METHOD_BIT_PARALLEL_64 = 3,
  MSBFS_METHOD_BIT_PARALLEL_64_PULL = 4,
  MSBFS_METHOD_BOOLEAN_REACHABILITY = 5,
  MSBFS_METHOD_PUSH_PULL_ADAPTIVE = 6,
  MSBFS_METHOD_SPARSE_QUEUE = 7,
  MSBFS_METHOD_SPARSE_BIT_PARALLEL_64 = 8,
  MSBFS_METHOD_MULTI_WORD_BIT_PARALLEL = 9,
  MSBFS_METHOD_INDIRECT_MACRO_BATCH = 10,
  MSBFS_METHOD_INDIRECT_SPARSE_QUEUE_PUSH = 11,
  MSBFS_METHOD_MULTI_WORD_BIT_PARALLEL_PUSH = 12,
  MSBFS_METHOD_WORKGROUP_PERSISTENT_BFS = 13,
  MSBFS_METHOD_AUTO = 14
} msbfs_method;

/* Kernel path a call actually ran (reported in msbfs_stats.path). */
#define MSBFS_PATH_NONE 0
#define MSBFS_PATH_PUSH 1   /* level-synchronous, top-down only            */
#define MSBFS_PATH_PULL 2   /* level-synchronous, bottom-up only           */
#define MSBFS_PATH_HYBRID 3 /* level-synchronous, device-decided direction */
#define MSBFS_PATH_CTA 4    /* one CTA per source, whole BFS in one launch */

typedef struct msbfs_engine msbfs_engine;
typedef struct msbfs_graph msbfs_graph;

/* Per-call statistics (filled when a non-NULL pointer is passed). */
typedef struct msbfs_stats {
  uint32_t method;           /* resolved msbfs_method                        */
  uint32_t path;             /* MSBFS_PATH_*                                 */
  uint32_t passes;           /* source chunks traversed                      */
  uint32_t words_per_vertex; /* u32 frontier words per vertex per pass       */
  uint32_t levels;           /* max BFS levels over passes                   */
  uint32_t push_levels;      /* summed over passes                           */
  uint32_t pull_levels;      /* summed over passes                           */
  uint32_t cta_cluster;      /* CTA path: blocks per cluster sharing a source's
                                visited bitmap (0: one block per source)     */
  uint64_t reached_pairs;    /* (s, v) pairs with a finite distance          */
  double gpu_ms;             /* device time of the whole call (CUDA events)  */
} msbfs_stats;

/* One record per launch of the level kernel (and one for the distance
 * materialisation), collected when profiling is on. Counters are those the
 * kernels keep for the algorithmic-bytes model; no reference counterpart
 * (the wgpu path has no timestamp queries, multi_word_bp.rs:762). */
#define MSBFS_DIR_TOP_DOWN 0
#define MSBFS_DIR_BOTTOM_UP 1
#define MSBFS_DIR_MATERIALIZE 2
typedef struct msbfs_level_record {
  uint32_t pass;
  uint32_t level;
  uint32_t dir;               /* MSBFS_DIR_*                               */
  uint32_t frontier_vertices; /* vertices in the level's input frontier    */
  uint64_t frontier_entries;  /* queue entries (hubs split into slices)    */
  uint64_t active;            /* bottom-up: vertex rows read               */
  uint64_t edges;             /* bottom-up: in-neighbour gathers;
                                 top-down: out-edges walked                */
  uint64_t new_vertices;      /* vertices that gained a visited lane       */
  uint64_t new_pairs;         /* (source, vertex) pairs discovered         */
  uint64_t rows;              /* bottom-up: frontier rows gathered (the
                                 in-neighbour was in the frontier)         */
  double device_ms;           /* %globaltimer span of the launch           */
  double event_ms;            /* CUDA-event span (profiling level 2) or 0  */
} msbfs_level_record;

/* Host-side CSR, mirroring CsrGraph (crates/core/src/graph.rs:8-22):
 * row_offsets[V+1], col_indices[E], u32, sorted and deduplicated rows.
 * Arrays returned by the library are malloc'd; release them with
 * msbfs_csr_free. The same struct carries a CscGraph (graph.rs:27-41) with
 * row_offsets = col_offsets and col_indices = row_indices. */
typedef struct msbfs_csr {
  size_t num_vertices;
  size_t num_edges;
  uint32_t *row_offsets;
  uint32_t *col_indices;
} msbfs_csr;

/* ======================= engine (crates/gpu_bfs) ========================== */

/* GpuBfsEngine::new (engine.rs:68-78): binds CUDA device `device` and fixes
 * the default method. */
int msbfs_engine_create(int device, int method, msbfs_engine **out);
void msbfs_engine_destroy(msbfs_engine *engine);
/* GpuBfsEngine::method (engine.rs:209-212). */
int msbfs_engine_method(const msbfs_engine *engine);
/* Text of the last error on this engine (anyhow message in the reference). */
const char *msbfs_engine_last_error(const msbfs_engine *engine);
/* Launch on a caller-owned cudaStream_t (NULL = the engine's own stream).
 * No reference counterpart: wgpu owns its queue. */
int msbfs_engine_set_stream(msbfs_engine *engine, void *cuda_stream);
/* Tuning knobs of the level-synchronous path (no reference counterpart; the
 * reference hard-codes alpha=14/beta=24 in push_pull.rs:29-36 and 512-source
 * chunks in multi_word_bp.rs:630). Zero keeps the current value. */
int msbfs_engine_set_tuning(msbfs_engine *engine, uint32_t max_words_per_pass,
                            uint32_t alpha, uint32_t beta);
/* Autotuner of the level-synchronous path. No single reference
 * counterpart: the reference fixes its thresholds -- alpha = 14 / beta = 24
 * for the direction switch (crates/gpu_bfs/src/dispatch/push_pull.rs:29-36),
 * the bottom-up density threshold of the hybrid prep kernel
 * (crates/shaders/src/prep_hybrid_hop.wgsl:67-71) and 512-source chunks
 * (crates/gpu_bfs/src/dispatch/multi_word_bp.rs:630) -- and picks a method
 * per call by fixed rules (engine.rs:157-198). For the graph's class
 * (road-like / mesh / power-law x vertex-count bucket, the batched form's
 * classes) and the source count rounded up to a power of two, the autotuner
 * times the call on the given sources (per-source statistics output, CUDA
 * events) while it varies one setting at a time over its candidates -- words
 * per vertex of a pass, alpha, beta, the in-edge slice length of bottom-up
 * steps, the frontier-bitmap threshold and the in-degree from which a whole
 * warp scans a vertex -- keeping a change only when it is
 * faster, then applies the best settings to the engine (and the slice length
 * to the graph). With a cache path, a class already in the file is applied
 * without timing and new classes are appended. Results never depend on the
 * settings. Calls that the router sends to the CTA-per-source path are not
 * tuned (the settings do not apply to it). */
typedef struct msbfs_tuning {
  uint32_t max_words_per_pass; /* u32 words per vertex of this call's passes       */
  uint32_t alpha;              /* top-down -> bottom-up: frontier out-edges * alpha > E */
  uint32_t beta;               /* bottom-up -> top-down: frontier vertices * beta < V  */
  uint32_t hub_split;          /* in-edge slice length of bottom-up steps              */
  uint32_t bitmap_div;         /* frontier-bitmap test below V / bitmap_div vertices    */
  uint32_t warp_scan_degree;   /* in-degree from which a whole warp scans a vertex      */
  uint32_t from_cache;         /* 1: read from the cache file, not timed               */
  uint32_t trials;             /* settings timed                                        */
  uint32_t level_path;         /* 0: the call runs on the CTA path, nothing tuned       */
  double ms;                   /* device time of one call with the chosen settings     */
  double default_ms;           /* the same with the settings the engine had before     */
  char class_name[48];         /* graph class and source bucket, "powerlaw/v2^22/s512" */
} msbfs_tuning;
int msbfs_engine_autotune(msbfs_engine *engine, msbfs_graph *graph, const uint32_t *sources,
                          size_t num_sources, const char *cache_path, msbfs_tuning *out);

/* Caps the persistent kernels' grids at `percent` (1..100, default 100) of
 * the blocks that fit the device at once, leaving the rest of the SMs to
 * kernels of other streams (the served form gives them to its express
 * slots). No reference counterpart. Results do not depend on it. */
int msbfs_engine_set_sm_share(msbfs_engine *engine, uint32_t percent);

/* Caps the levels of one level-synchronous pass (0, the default, = V + 2,
 * which no traversal reaches). A pass still running at the cap stops, its
 * buffers are cleared as after a normal stop, and the call returns
 * MSBFS_ERR_TIMEOUT ("level cap reached"); the engine stays usable. The
 * reference bounds its hop loop at V hops and, if that runs out, returns the
 * rows it has without an error (crates/gpu_bfs/src/dispatch/
 * indirect_sparse_push.rs:1463-1577); here partial rows are never reported as
 * a success. The CTA-per-source path ends after at most V levels by
 * construction and ignores the cap. */
int msbfs_engine_set_level_cap(msbfs_engine *engine, uint32_t max_levels);

/* Profiling: 0 off; 1 keep a per-level record of every call (device timers
 * and the work counters of the algorithmic-bytes model; the level loop stays
 * on the device and runs the level kernels' counting form); 2 as 1, but the
 * level loop is driven from the host one launch at a time with CUDA events
 * around each launch; 3 as 2 with the production level kernels, which keep
 * no work counters (the records carry durations, frontier sizes and
 * discovered pairs only). msbfs_engine_level_log copies the last call's
 * records. */
int msbfs_engine_set_profiling(msbfs_engine *engine, int level);
int msbfs_engine_level_log(const msbfs_engine *engine, msbfs_level_record *out,
                           size_t capacity, size_t *count);

/* GpuBfsEngine::select_auto_method (engine.rs:157-198), same branches:
 * empty graph or S == 0 -> NAIVE_SEQUENTIAL; max_degree <= 8 && E <= 4V ->
 * WORKGROUP_PERSISTENT_BFS; max_degree >= 128 -> INDIRECT_SPARSE_QUEUE_PUSH;
 * else S >= 64 -> MULTI_WORD_BIT_PARALLEL, S >= 32 -> BIT_PARALLEL_64,
 * S > 1 -> BIT_PARALLEL_32, S == 1 -> SPARSE_QUEUE. */
int msbfs_select_auto_method(size_t num_vertices, size_t num_edges,
                             const uint32_t *row_offsets, size_t num_sources);

/* Uploads a CsrGraph and keeps it resident in HBM: CSR for top-down steps
 * and its transpose (CSC) for bottom-up steps, aliased when the graph is
 * symmetric (PushPullGraphBuffers::from_symmetric_graph / from_graph,
 * crates/gpu_bfs/src/buffer.rs:108-221). The arrays are validated like
 * CsrGraph::validate (graph.rs:226-280) and copied; the caller keeps
 * ownership. */
int msbfs_graph_create(msbfs_engine *engine, size_t num_vertices,
                       size_t num_edges, const uint32_t *row_offsets,
                       const uint32_t *col_indices, msbfs_graph **out);
void msbfs_graph_destroy(msbfs_graph *graph);
/* Graph facts used by the router: V, E, max out-degree, symmetric flag. */
int msbfs_graph_info(const msbfs_graph *graph, size_t *num_vertices,
                     size_t *num_edges, uint32_t *max_degree,
                     int *is_symmetric);

/* BfsEngine::run_ms_bfs / GpuBfsEngine::run_ms_bfs_into (crates/core/src/
 * lib.rs:38, engine.rs:219-298) with the engine's method (AUTO resolves per
 * call). `out` is caller-owned HOST memory of S*V u32. S == 0 writes nothing
 * and succeeds; V == 0 with S > 0 is MSBFS_ERR_EMPTY_GRAPH; a source >= V is
 * MSBFS_ERR_SOURCE_OOB and nothing is written. Blocks until `out` is filled. */
int msbfs_run_ms_bfs(msbfs_engine *engine, const msbfs_graph *graph,
                     const uint32_t *sources, size_t num_sources,
                     uint32_t *out, msbfs_stats *stats);

/* GpuBfsEngine::run_ms_bfs_with_method (engine.rs:300-405). */
int msbfs_run_ms_bfs_with_method(msbfs_engine *engine, int method,
                                 const msbfs_graph *graph,
                                 const uint32_t *sources, size_t num_sources,
                                 uint32_t *out, msbfs_stats *stats);

/* One-shot form of BfsEngine::run_ms_bfs(&CsrGraph, &[u32]) for callers that
 * hold only host CSR arrays: uploads the graph for this call, runs, frees. */
int msbfs_run_ms_bfs_csr(msbfs_engine *engine, size_t num_vertices,
                         size_t num_edges, const uint32_t *row_offsets,
                         const uint32_t *col_indices, const uint32_t *sources,
                         size_t num_sources, uint32_t *out, msbfs_stats *stats);

/* Device-resident form of run_ms_bfs_into: `out_device` is a device pointer
 * to S*V u32. Work is queued on the engine's stream and the call returns
 * without waiting; msbfs_engine_synchronize waits and fills `stats`. Sources
 * are validated on the host before anything is queued. No reference
 * counterpart (the wgpu path always reads back to the host). */
int msbfs_run_ms_bfs_device(msbfs_engine *engine, int method,
                            const msbfs_graph *graph, const uint32_t *sources,
                            size_t num_sources, uint32_t *out_device);
int msbfs_engine_synchronize(msbfs_engine *engine, msbfs_stats *stats);

/* Per-source reductions instead of distance rows (served form output; no
 * reference counterpart): eccentricity = largest finite distance, reached =
 * vertices with a finite distance (the source included), distance_sum = sum
 * of finite distances. Computed on the device from the traversal state; the
 * S*V matrix is never formed. */
typedef struct msbfs_source_stats {
  uint64_t distance_sum;
  uint32_t eccentricity;
  uint32_t reached;
} msbfs_source_stats;
/* Device output, queued without waiting (msbfs_engine_synchronize waits). */
int msbfs_run_ms_bfs_stats_device(msbfs_engine *engine, int method,
                                  const msbfs_graph *graph, const uint32_t *sources,
                                  size_t num_sources,
                                  msbfs_source_stats *stats_device);
/* Host output, blocking, engine's method. */
int msbfs_run_ms_bfs_stats(msbfs_engine *engine, const msbfs_graph *graph,
                           const uint32_t *sources, size_t num_sources,
                           msbfs_source_stats *out, msbfs_stats *stats);

/* ===================== served form (resident graph, request stream) ======
 * No reference counterpart (the reference is one blocking call per query).
 * A server keeps the graph resident and runs `slots` traversals at once,
 * each on its own engine and stream. A scheduler thread packs queued
 * requests of the same output mode into the next free slot's launch --
 * unrelated requests share the source lanes of one traversal -- so requests
 * arriving while others run are admitted as slots free up and their work
 * overlaps on the device. Admission is by device bytes: each slot's
 * traversal state is allocated once, and distance rows are staged in one
 * pool of hbm_budget_bytes shared by all slots; a launch of rows requests
 * takes only as many lanes as the pool's largest free range holds rows for
 * (V u32 per lane), reserves those bytes and returns them when it completes,
 * so a request needing more rows than are free is split across launches.
 * Every result is the same bytes as a lone msbfs_run_ms_bfs /
 * msbfs_run_ms_bfs_stats call.
 *
 * Latency: a request of at most small_sources sources is "small". The first
 * express_slots slots take only small requests (at most 2*small_sources
 * lanes per launch, so their traversals stay narrow) on the device's
 * highest-priority streams; the other slots take large requests first, in
 * arrival order, and small ones only when no large request waits. Their
 * persistent kernels use general_sm_percent of the resident grid
 * (msbfs_engine_set_sm_share) so express kernels find SMs free. */
#define MSBFS_SERVE_ROWS 0  /* out = S*V u32 distance rows          */
#define MSBFS_SERVE_STATS 1 /* out = S msbfs_source_stats           */
typedef struct msbfs_server msbfs_server;
typedef struct msbfs_server_config {
  uint32_t slots;                  /* traversals in flight (0 -> 2)            */
  uint32_t max_sources_per_launch; /* lanes packed per launch (0 -> 512); above
                                      512, general slots run each launch as one
                                      pass of up to 64 words (2,048 lanes)    */
  uint64_t hbm_budget_bytes;       /* row pool of all slots (0 -> 8 GiB)       */
  int method;                      /* engine method (MSBFS_METHOD_AUTO)        */
  uint32_t express_slots;          /* slots reserved for small requests (0)    */
  uint32_t small_sources;          /* small-request threshold (0 -> 64)        */
  uint32_t general_sm_percent;     /* grid share of the other slots (0 -> 100) */
  uint32_t reserved;               /* must be 0                                */
} msbfs_server_config;
/* Totals since creation: traversals launched and kernel launches (level
 * loop launches counted from each traversal's level count). */
int msbfs_server_counters(msbfs_server *server, uint64_t *traversals,
                          uint64_t *kernel_launches);
typedef struct msbfs_request_info {
  double latency_ms; /* submit -> result in host memory       */
  double queue_ms;   /* submit -> first launch                */
  uint32_t launches; /* launches the request was split into   */
  int status;        /* MSBFS_OK or an error code             */
} msbfs_request_info;
int msbfs_server_create(int device, size_t num_vertices, size_t num_edges,
                        const uint32_t *row_offsets, const uint32_t *col_indices,
                        const msbfs_server_config *config, msbfs_server **out);
/* Queues a request; `sources` is copied, `out` (host, S*V u32 or S stats)
 * must stay valid until the request completes. Returns a ticket. */
int msbfs_server_submit(msbfs_server *server, const uint32_t *sources,
                        size_t num_sources, int mode, void *out, uint64_t *ticket);
/* Waits for a ticket (timeout_ms < 0: forever); MSBFS_ERR_TIMEOUT if it
 * did not complete in time. The ticket is released once it has completed. */
int msbfs_server_wait(msbfs_server *server, uint64_t ticket, double timeout_ms,
                      msbfs_request_info *info);
void msbfs_server_destroy(msbfs_server *server);

/* GpuBfsEngine::run_ms_reachability (engine.rs:420-479): HOST words of
 * V * ceil(S/32) u32, words[v * wpv + s / 32] bit (s % 32) set iff v is
 * reachable from sources[s] (ReachabilityBitmask, graph.rs:446-452). */
int msbfs_run_reachability(msbfs_engine *engine, const msbfs_graph *graph,
                           const uint32_t *sources, size_t num_sources,
                           uint32_t *words, msbfs_stats *stats);

/* Traversed edges of a result, sum over s of out-degrees of reached vertices
 * (crates/cli/src/bench.rs:478-491), computed on the device from a
 * device-resident distance matrix. */
int msbfs_traversed_edges_device(msbfs_engine *engine, const msbfs_graph *graph,
                                 const uint32_t *dist_device,
                                 size_t num_sources, uint64_t *out_edges);

/* ------------------------------------------------------------------------
 * Multi-source BFS that allocates nothing. No counterpart in the reference.
 *
 * For callers that must not call cudaMalloc: host applications that hand all
 * device memory to their own pool allocator and do not let libraries
 * allocate beside it, and services that reserve every byte they will use
 * when they start, so that no request can fail later for want of memory.
 * Every other entry point allocates engine-owned device buffers; this one
 * uses no engine. It runs the one-block-per-source BFS (the kernel behind
 * MSBFS_METHOD_WORKGROUP_PERSISTENT_BFS) with its scratch -- a copy of the
 * sources, the source cursor and one frontier queue slab of V u32 per
 * resident block -- in a fixed device array of MSBFS_NOALLOC_SCRATCH_BYTES
 * inside the library. Every GPU that loads the library holds that array
 * until the process exits.
 *
 * Inputs and outputs stay the caller's: the CSR arrays and the S*V u32
 * distance matrix are DEVICE pointers (dist[s*V + v], unreachable =
 * 0xFFFFFFFF, the same bytes as msbfs_run_ms_bfs); `sources` is a HOST array,
 * validated like msbfs_run_ms_bfs (MSBFS_ERR_SOURCE_OOB) and copied into the
 * fixed array with cudaMemcpyAsync on `cuda_stream`: from pageable memory the
 * copy is staged before the call returns, from page-locked memory it runs in
 * stream order, so such an array must stay unchanged until the stream has
 * passed this call. Work is queued on `cuda_stream` (NULL = legacy default
 * stream) and the call returns without waiting. Calls of more than 65,536
 * sources run as consecutive chunks of at most that many. Graphs with more
 * than MSBFS_NOALLOC_MAX_VERTICES vertices are rejected with
 * MSBFS_ERR_SCRATCH_TOO_SMALL before anything is queued.
 *
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture begins. The calling thread's current device is restored before
 * the call returns, and a CUDA error left pending on the thread by earlier
 * work is cleared before this call queues its own, so MSBFS_ERR_CUDA reports
 * this call's failures only. All calls share the one array, which keeps the
 * last call's contents (the cursor is cleared by each call): calls that
 * overlap on the GPU -- on different streams, or before the previous call's
 * work finished on another stream -- race on it and must be serialised by
 * the caller. */
#define MSBFS_NOALLOC_SCRATCH_BYTES (32u << 20)
#define MSBFS_NOALLOC_MAX_VERTICES 1048576u
int msbfs_run_cta_noalloc(int device, size_t num_vertices,
                          const uint32_t *row_offsets_device,
                          const uint32_t *col_indices_device,
                          const uint32_t *sources, size_t num_sources,
                          uint32_t *dist_device, void *cuda_stream);

/* ===================== graph core (crates/core) =========================== */

void msbfs_csr_free(msbfs_csr *csr);
/* CsrGraph::from_edge_list (graph.rs:51-79): drops self-loops and
 * out-of-range endpoints, sorts by (u, v) and deduplicates. */
int msbfs_csr_from_edge_list(size_t num_vertices, size_t num_pairs,
                             const uint32_t *src, const uint32_t *dst,
                             msbfs_csr *out);
/* CsrGraph::to_csc (graph.rs:90-127); also CscGraph::to_csr (graph.rs:
 * 283-316), which is the same counting-sort transpose. */
int msbfs_csr_transpose(const msbfs_csr *in, msbfs_csr *out);
/* CsrGraph::is_symmetric (graph.rs:129-133): 1 / 0. */
int msbfs_csr_is_symmetric(const msbfs_csr *csr);
/* CsrGraph::to_undirected (graph.rs:136-151). */
int msbfs_csr_to_undirected(const msbfs_csr *in, msbfs_csr *out);
/* CsrGraph::validate (graph.rs:226-280); message written to `msg`. */
int msbfs_csr_validate(const msbfs_csr *csr, char *msg, size_t msg_len);
/* CsrGraph::max_degree (graph.rs:209-214). */
uint32_t msbfs_csr_max_degree(const msbfs_csr *csr);

/* ==================== Matrix Market reader (crates/core/src/mtx.rs) ========
 * MtxReader::parse (mtx.rs:124-275): coordinate format only; pattern, real,
 * integer or complex fields (values ignored); symmetric, skew-symmetric and
 * hermitian matrices must be square and are expanded to both directions;
 * 1-based indices; self-loops dropped; V = max(rows, cols); adjacency sorted
 * and deduplicated. On MSBFS_ERR_PARSE, `err` (optional) holds the MtxError
 * variant (crates/core/src/error.rs:43-81), its fields and its message. */
#define MSBFS_MTX_OK 0
#define MSBFS_MTX_IO 1
#define MSBFS_MTX_INVALID_HEADER 2
#define MSBFS_MTX_UNSUPPORTED_FORMAT 3
#define MSBFS_MTX_INVALID_DIMENSIONS 4
#define MSBFS_MTX_INVALID_COORDINATE_LINE 5
#define MSBFS_MTX_ZERO_INDEX 6
#define MSBFS_MTX_INDEX_OUT_OF_BOUNDS 7
typedef struct msbfs_mtx_error {
  int kind;              /* MSBFS_MTX_*                                  */
  uint64_t line_number;  /* 1-based line of the offending text (0: none) */
  uint64_t row, col;     /* ZERO_INDEX / INDEX_OUT_OF_BOUNDS entry        */
  uint64_t max_rows, max_cols;
  char message[256];     /* the reference's error text                   */
} msbfs_mtx_error;
int msbfs_mtx_parse(const char *text, size_t len, msbfs_csr *out, msbfs_mtx_error *err);
int msbfs_mtx_read(const char *path, msbfs_csr *out, msbfs_mtx_error *err);

/* ==================== generators (crates/core/src/generators.rs) ==========
 * Seeded with the engine's own counter-based generator (splitmix64), so the
 * bytes differ from the reference's rand::StdRng for the same seed; the
 * structural rules (symmetrised, sorted, deduplicated, no self-loops) are the
 * reference's. */
/* Grid2D::new (generators.rs:28-80): N, W, E, S neighbour order. */
int msbfs_gen_grid2d(size_t width, size_t height, msbfs_csr *out);
/* generate_erdos_renyi_np (generators.rs:139-191), geometric skipping. */
int msbfs_gen_erdos_renyi_np(size_t n, double p, uint64_t seed, msbfs_csr *out);
/* generate_random_tree (generators.rs:239-262): uniform recursive tree over
 * a shuffled vertex order. */
int msbfs_gen_random_tree(size_t n, uint64_t seed, msbfs_csr *out);
/* generate_rmat (generators.rs:277-342): quadrant recursion, self-loops
 * dropped, symmetrised unless `directed`. Multi-threaded; the output does not
 * depend on the thread count. */
int msbfs_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                   double c, double d, uint64_t seed, int directed,
                   msbfs_csr *out);
/* path_graph, star_graph, cycle_graph, clique_graph, disconnected_cliques
 * (generators.rs:388-544). */
int msbfs_gen_path(size_t n, msbfs_csr *out);
int msbfs_gen_star(size_t n, msbfs_csr *out);
int msbfs_gen_cycle(size_t n, msbfs_csr *out);
int msbfs_gen_clique(size_t n, msbfs_csr *out);
int msbfs_gen_disconnected_cliques(const size_t *sizes, size_t count,
                                   msbfs_csr *out);
/* Road-like graph (no reference counterpart): a uniform spanning tree of the
 * width x height 4-neighbour grid drawn with Wilson's algorithm, plus
 * `extra_edges` distinct grid edges not in the tree, symmetrised. */
int msbfs_gen_wilson_grid(size_t width, size_t height, size_t extra_edges,
                          uint64_t seed, msbfs_csr *out);
/* sample_sources, random strategy (crates/cli/src/graph_loader.rs:132-190):
 * `count` distinct vertices drawn uniformly without replacement among those
 * with out-degree >= min_degree, returned sorted ascending. */
int msbfs_sample_sources(const msbfs_csr *csr, size_t count, uint64_t seed,
                         uint32_t min_degree, uint32_t *out);

/* ===================== batched form (many graphs, one launch) =============
 * No single reference counterpart: the reference traverses one graph per
 * GpuBfsEngine call (engine.rs:219) with fixed method thresholds
 * (engine.rs:157-198). A batch uploads many graphs with their sources once;
 * msbfs_batch_run traverses all of them in ONE persistent kernel launch that
 * pulls (graph, source range) items from a device work list. Per graph class
 * (road-like / mesh / power-law x vertex-count bucket) the autotuner times
 * candidate configurations (block-synchronous bit-parallel BFS with 1-8
 * words per vertex, three bottom-up thresholds and two tile shapes -- a
 * thread per vertex word, or a thread per vertex holding all its words --
 * or one single-source BFS per source with 1/4/16 sources per item) on
 * sample graphs of that class
 * and caches the fastest, optionally in a text file. Results (S*V u32 per
 * graph, same bytes as msbfs_run_ms_bfs) stay in device memory until read. */
#define MSBFS_BATCH_MAX_VERTICES 262144u
typedef struct msbfs_batch msbfs_batch;
typedef struct msbfs_batch_graph {
  size_t num_vertices;
  size_t num_edges;
  const uint32_t *row_offsets; /* CSR, validated like CsrGraph::validate */
  const uint32_t *col_indices;
  const uint32_t *sources;     /* host, each < num_vertices */
  size_t num_sources;
} msbfs_batch_graph;
int msbfs_batch_create(int device, const msbfs_batch_graph *graphs, size_t num_graphs,
                       msbfs_batch **out);
void msbfs_batch_destroy(msbfs_batch *batch);
int msbfs_batch_autotune(msbfs_batch *batch, size_t samples_per_class,
                         const char *cache_path);
/* One persistent launch over every graph; device time in *gpu_ms. */
int msbfs_batch_run(msbfs_batch *batch, double *gpu_ms);
/* The plain comparison: one msbfs_run_ms_bfs_device call per graph (Auto
 * method), same outputs; `graphs` must be the array given at creation. */
int msbfs_batch_run_per_graph(msbfs_batch *batch, const msbfs_batch_graph *graphs,
                              double *gpu_ms);
/* Copies graph i's S*V distance rows to host memory. */
int msbfs_batch_result(msbfs_batch *batch, size_t graph_index, uint32_t *out);
/* The tuned configuration of graph i's class: alg 0 = bit-parallel block
 * with a thread per vertex word, 2 = the same with a thread per vertex
 * (words = max words per vertex, param = bottom-up divisor for both),
 * 1 = one source per BFS (param = sources per item). */
int msbfs_batch_config(const msbfs_batch *batch, size_t graph_index, uint32_t *alg,
                       uint32_t *words, uint32_t *param, char *class_name,
                       size_t class_len);

#ifdef __cplusplus
}
#endif

#endif /* MSBFS_H */
