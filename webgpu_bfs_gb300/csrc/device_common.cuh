// Device-side data structures shared by the level-synchronous kernels, the
// CTA-per-source kernel and the host orchestration (engine.cu).
//
// HBM layout of one level-synchronous pass over P <= 32*W sources:
//   vis[V][W]        u32 visited bits, lane s of word s/32 = source s of the pass
//   F[3][V][W]       frontier words, rotated by level: level L reads F[L%3],
//                    writes F[(L+1)%3] and clears F[(L+2)%3] (= level L-1)
//   planes[NP][V][W] bit-sliced discovery levels: bit b of d(s,v) is stored
//                    in lane s of planes[b][v][s/32]; materialised into the
//                    source-major u32 distance matrix once, after the loop
//   ovf[V][W]        lanes whose distance did not fit NP planes; those were
//                    written straight into the distance matrix
//   Q[3][qcap]       u64 queue entries (seg << 32 | v): frontier vertices, one
//                    entry per SEG out-edges so hub expansion is split (Q[0]
//                    holds V + E/SEG0 entries: the sources' queue uses SEG0)
//   stamp[V]         level at which v was last enqueued by a top-down step
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace msbfs {

enum : uint32_t { DIR_PUSH = 0, DIR_PULL = 1 };
enum : uint32_t { MODE_PUSH = 1, MODE_PULL = 2, MODE_HYBRID = 3 };
enum : uint32_t { STATUS_LEVEL_CAP = 1u, STATUS_BAD_SOURCE = 2u, STATUS_CHECK = 4u };

// Per-level record written by the level controller (counters feed the
// algorithmic-bytes model of the roofline; t is %globaltimer ns).
struct LevelRec {
  uint32_t level;
  uint32_t dir;
  uint32_t frontier_vertices;  // |Q_L| vertices
  uint32_t frontier_entries;   // |Q_L| entries (hub vertices split by seg)
  unsigned long long active;   // bottom-up: vertex rows read (in-degree > 0)
  unsigned long long edges;    // bottom-up: in-neighbour gathers; top-down: out-edges walked
  unsigned long long new_vertices;
  unsigned long long new_pairs;
  unsigned long long rows;     // frontier rows gathered (bottom-up)
  unsigned long long t_start;
  unsigned long long t_end;
};

constexpr uint32_t LOG_CAP = 4096;
constexpr uint32_t WORK_STRIPES = 16;

struct LevelCtl {
  uint32_t level;      // frontier level L being expanded
  uint32_t dir;        // direction of level L
  uint32_t terminated; // 1 once a level discovered nothing
  uint32_t status;     // STATUS_* bits
  uint32_t qcount[4];  // queue entries per slot (slot 3 unused)
  uint32_t qverts[4];  // vertices per slot
  unsigned long long qedges[4];  // sum of out-degrees per slot
  unsigned long long explored;   // out-edges of all expanded frontiers
  unsigned long long pairs;      // discovered (s, v) pairs, sources included
  uint32_t done_blocks;          // last-block-done counter of the level kernel
  uint32_t push_levels;
  uint32_t pull_levels;
  uint32_t check_site;           // bounds-checked build: first failed check site
  unsigned long long c_active;   // counters of the running level
  unsigned long long c_edges;
  unsigned long long c_newv;
  unsigned long long c_pairs;
  unsigned long long c_rows;
  unsigned long long t_start;    // min %globaltimer over the level's blocks
  uint32_t use_bits;             // bottom-up step checks frontier bitmaps first
  uint32_t narrow;               // the pass's rows went to PassDesc::dist8 as bytes
  // Vertex-tile cursors of the running bottom-up step: the work list is cut
  // into WORK_STRIPES contiguous stripes, each with its own cursor on its own
  // 128-byte line, so the claims of a level spread over several L2 slices
  // instead of queueing on one address.
  alignas(128) uint32_t work[WORK_STRIPES][32];

  // Source lanes whose frontier is non-empty: lanes[L & 1] for the level being
  // expanded, lanes[(L + 1) & 1] collects the lanes that gain vertices. A lane
  // with an empty frontier can discover nothing, so bottom-up steps ignore it.
  uint32_t lanes[2][64];
};

// One slice of a high in-degree vertex's in-edge list, scanned by one warp
// during bottom-up steps; the last slice to finish records the result.
struct HeavyChunk {
  uint32_t v;      // vertex
  uint32_t j;      // slice index
  uint32_t nch;    // slices of this vertex
  uint32_t h;      // index of the vertex among heavy vertices
};

// Per-pass descriptor, read from device memory so one captured CUDA graph can
// serve every pass and every call.
// Per-source reductions of a traversal (served form): eccentricity (largest
// finite distance), reached vertices (the source included) and the sum of
// finite distances. Layout shared with msbfs_source_stats in msbfs.h.
struct SourceStats {
  unsigned long long sum;
  uint32_t ecc;
  uint32_t reached;
};

struct PassDesc {
  const uint32_t* sources;  // this pass's sources (device)
  uint32_t* dist;           // first row of this pass in the distance matrix
  uint32_t* reach;          // non-null: write visited words here instead
  SourceStats* stats;       // non-null: per-source reductions instead of rows
  // Non-null: when every distance of the pass is below 255, the rows are
  // written here as one byte per distance (0xFF = unreachable) instead of
  // into `dist`, and LevelCtl::narrow is set; the host widens them.
  uint8_t* dist8;
  uint32_t num_sources;     // P
  uint32_t reach_wpv;       // words per vertex of the reachability output
  uint32_t reach_col;       // word column of this pass in that output
  uint32_t row_split;       // split materialisation: rows below go u32 to dist,
                            // rows from it on as bytes to dist8 (multiple of 32)
};

struct LevelParams {
  uint32_t V;
  uint32_t W;        // u32 words per vertex (template argument, repeated)
  unsigned long long E;
  const uint32_t* out_off;  // CSR: top-down steps
  const uint32_t* out_idx;
  const uint32_t* in_off;   // CSC: bottom-up steps (aliases CSR if symmetric)
  const uint32_t* in_idx;
  uint32_t* vis;
  uint32_t* F[3];
  uint32_t* planes;
  uint32_t* ovf;
  unsigned long long* Q[3];
  uint32_t* stamp;
  uint32_t* fbits[3];  // frontier membership bitmaps (V bits), rotated like F
  LevelCtl* ctl;
  LevelRec* log;      // LOG_CAP records
  const PassDesc* desc;
  uint32_t NP;        // planes allocated
  uint32_t qcap;      // entries per queue slot (slots 1, 2)
  uint32_t qcap0;     // entries of slot 0 (the sources' queue uses shorter entries)
  uint32_t mode;      // MODE_*
  uint32_t alpha;     // push -> pull when m_f * alpha > unexplored edges
  uint32_t beta;      // pull -> push when n_f * beta < V
  uint32_t seg;       // out-edges per queue entry
  uint32_t seg0;      // out-edges per entry of the sources' queue (level 0)
  uint32_t heavy;     // in-degree from which a whole warp scans one vertex
  uint32_t max_levels;
  uint32_t split;     // in-degree above which in-edges are sliced across warps
  uint32_t n_hchunks;
  const HeavyChunk* hchunks;
  uint32_t* hcand;    // [n_heavy][W] candidate words of sliced vertices
  uint32_t* hcount;   // [n_heavy] slices finished this level
  // Bit ci: the vertex of slice ci may still need lanes. Set at pass start,
  // cleared for good once the slice finds none needed (a vertex's needed
  // lanes only shrink: visited lanes grow, live lanes die).
  uint32_t* hlive;
  uint32_t hlive_words;
  uint32_t bits_div;  // bitmap check when the frontier holds < V / bits_div vertices
  uint32_t n_order;
  const uint4* order;  // {v, in-edge begin, end, 0} for 0 < in-degree <= split (work order)
};

// Launch helpers implemented in level_kernels.cu / cta_kernel.cu.
struct LevelKernelInfo {
  void* init;         // kernel symbols for graph nodes
  void* level[2][2];  // [direction: DIR_PUSH, DIR_PULL][with profiling counters]
  int level_grids[2]; // resident grid per direction
  void* materialize;
  void* reduce;       // per-source reductions in place of materialize
  void* cleanup;
  int level_block;
  int mat_block;
  int mat_grid;
  size_t mat_smem;
  int red_block;
  int red_grid;
};
// Fills kernel symbols and launch shapes for words-per-vertex W and NP level
// planes (the materialisation stages 1 + NP arrays in shared memory).
bool level_kernel_info(uint32_t W, uint32_t NP, int num_sms, LevelKernelInfo* out);
size_t materialize_smem_bytes(uint32_t W, uint32_t NP);
// (vertex tile, word group) items of a materialisation over V vertices at
// W words per vertex: an upper bound on what a pass of fewer sources uses.
size_t materialize_items(uint32_t V, uint32_t W);
void launch_init(const LevelParams& p, cudaStream_t s);
// Launches the level kernel of direction `dir` (DIR_PUSH / DIR_PULL), or
// both (pull, then push) when dir is DIR_BOTH; `count` picks the form that
// keeps the profiling counters.
constexpr uint32_t DIR_BOTH = 2;
void launch_level(const LevelParams& p, const LevelKernelInfo& k, uint32_t dir, bool count,
                  cudaStream_t s);
// reduce: per-source reductions (reduce_kernel) instead of rows or bitmasks.
// phase (materialisation only): MAT_ALL writes every row (bytes when the
// pass allows) and clears the traversal state; MAT_BYTES writes only the
// byte rows from PassDesc::row_split on and clears nothing (nothing at all
// unless every distance fits a byte); MAT_WIDE then writes the u32 rows
// below the split (all rows when the pass did not go to bytes) and clears.
enum : uint32_t { MAT_BYTES = 0, MAT_WIDE = 1, MAT_ALL = 2 };
void launch_materialize(const LevelParams& p, const LevelKernelInfo& k, bool reduce,
                        cudaStream_t s, uint32_t phase = MAT_ALL);
void launch_cleanup(const LevelParams& p, cudaStream_t s);

struct CtaParams {
  uint32_t V;
  const uint32_t* off;
  const uint32_t* idx;
  const uint32_t* sources;
  uint32_t num_sources;
  uint32_t* dist;        // row s at dist + s * V (null when stats is set)
  uint32_t* gqueue;      // per resident block: V u32
  uint32_t* work;        // source cursor (zeroed before launch)
  SourceStats* stats;    // non-null: per-source reductions instead of rows
  uint32_t* gbits;       // global-bitmap mode: per resident block ceil(V/32) u32
  uint32_t qh;           // frontier entries per shared-memory queue half (set at launch)
  const uint4* erec;     // per edge {target, target's edge begin, end, 0}, or null
};
struct CtaShape {
  int grid = 0;           // resident blocks
  int block = 0;          // threads per block
  size_t smem = 0;        // dynamic shared memory: bitmap (shared mode) + queue halves
  uint32_t qh = 0;        // frontier entries per shared-memory queue half
  int minb = 3;           // register budget: resident blocks per SM it is built for
  bool global_bits = false;
  bool edge_records = false;
  int cluster = 0;        // > 1: blocks per cluster sharing one source's bitmap
};
// Max V for the shared-memory visited bitmap; launch shape of the CTA kernel
// for a call of num_sources sources (above that V when allow_global: the
// bitmap split over the shared memory of a thread-block cluster for calls of
// few sources, an L2-resident global slab per block otherwise; edge-range
// queue entries when the graph has edge records). In cluster mode `grid`
// counts blocks (a multiple of `cluster`) and each cluster has one queue slab.
size_t cta_max_vertices(int device);
bool cta_launch_shape(uint32_t V, int device, bool allow_global, bool edge_records,
                      size_t num_sources, CtaShape* out);
void launch_cta(const CtaParams& p, const CtaShape& sh, int grid, cudaStream_t s);
void launch_edge_records(uint32_t V, const uint32_t* off, const uint32_t* idx, uint4* erec,
                         cudaStream_t s);

void launch_traversed_edges(uint32_t V, const uint32_t* off, const uint32_t* dist,
                            uint32_t num_sources, unsigned long long* out, cudaStream_t s);

}  // namespace msbfs
