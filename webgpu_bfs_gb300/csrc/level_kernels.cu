// Level-synchronous bit-parallel multi-source BFS kernels for sm_103a.
//
// One pass traverses up to 32*W sources at once: lane s of word s/32 of a
// vertex's W-word row belongs to source s. A level is one launch of
// level_kernel<W, DIR>, a bottom-up (pull) or a top-down (push) step, as
// decided on the device by the previous level; the loop itself is a
// CUDA-graph WHILE node whose condition the last block of each level sets.
//
// Semantics follow the reference's WGSL kernels:
//   bottom-up step  crates/shaders/src/multi_word_bp_pull_512.wgsl:69-138
//                   (needed = ~vis & mask; cand = OR of in-neighbours' frontier
//                   words with early exit once cand covers needed;
//                   newly = cand & needed)
//   top-down step   crates/shaders/src/indirect_sparse_push_512.wgsl:89-321
//                   (needed = f & ~vis; prev = atomicOr(vis, needed);
//                   newly = needed & ~prev; one enqueue per vertex per level)
//   direction       crates/shaders/src/prep_hybrid_hop.wgsl:46-134 and the
//                   host alpha/beta rule of crates/gpu_bfs/src/dispatch/
//                   push_pull.rs:484-498
//   source init     crates/shaders/src/init_sparse_push_sources_512.wgsl:27-67
// The GB300 design (vectorised 16-byte frontier gathers per lane group, a
// warp per heavy vertex, warp-aggregated atomics, block-staged queue
// compaction, bit-sliced level planes materialised into coalesced rows) is
// this file's own.
#include <cooperative_groups.h>

#include "device_common.cuh"

namespace msbfs {

#ifndef MSBFS_LEVEL_BLOCK
#define MSBFS_LEVEL_BLOCK 256
#endif
constexpr int LEVEL_BLOCK = MSBFS_LEVEL_BLOCK;
constexpr int BQ_CAP = 2048;  // discovered vertices staged per block
#ifndef MSBFS_PULL_CH
#define MSBFS_PULL_CH 4
#endif
#ifndef MSBFS_LEVEL_MIN_BLOCKS
// 8 resident blocks of 256 threads (all 64 warps of an SM, 32 registers):
// the bottom-up gathers are latency-bound, and the extra warps outweigh the
// spilled registers (R-MAT scale 22, S=512: dense levels 2.29 -> 1.92 ms
// against 6 blocks at 40 registers; 4 and 5 blocks were slower still).
#define MSBFS_LEVEL_MIN_BLOCKS (2048 / MSBFS_LEVEL_BLOCK)
#endif
constexpr int CH = MSBFS_PULL_CH;  // in-neighbours gathered per chunk
constexpr int MAT_BLOCK = 256;
constexpr uint32_t FULL = 0xffffffffu;
constexpr uint32_t DIST_MAX = 0xffffffffu;

// Bounds-checked build (-DMSBFS_BOUNDS_CHECK, the sanitizer's stand-in): an
// index outside its buffer, or a loop past its iteration limit, records the
// check's site id and STATUS_CHECK in the control block and skips the access
// (or leaves the loop) instead of faulting or running on; the host turns it
// into MSBFS_ERR_CUDA naming the site. The default build compiles the
// checks out.
#ifdef MSBFS_BOUNDS_CHECK
__device__ __noinline__ void check_fail(LevelCtl* c, uint32_t site) {
  atomicOr(&c->status, STATUS_CHECK);
  atomicCAS(&c->check_site, 0u, site);
}
#define BCHECK(ok, site) ((ok) ? true : (check_fail(p.ctl, (site)), false))
#define LOOP_GUARD(g, limit, site)  \
  if (++(g) > (limit)) {            \
    check_fail(p.ctl, (site));      \
    break;                          \
  }
#else
#define BCHECK(ok, site) true
#define LOOP_GUARD(g, limit, site)
#endif
// Check sites (reported by the host as "bounds check failed at site N").
enum : uint32_t {
  CK_TILE_LOOP = 1, CK_ORDER_ENTRY = 3, CK_GATHER_ID = 4, CK_SLICE = 5,
  CK_PUSH_ENTRY = 6, CK_PUSH_TARGET = 7, CK_CLEAR_ENTRY = 8, CK_QUEUE_CAP = 9
};

template <int W>
struct Geo {
  static constexpr int VEC = W >= 4 ? 4 : W;  // words per lane access
  static constexpr int LPV = W / VEC;         // lanes per vertex (a "group")
  static constexpr int GPW = 32 / LPV;        // groups per warp
};

template <int VEC>
struct Words {
  uint32_t w[VEC];
};

template <int VEC>
__device__ __forceinline__ Words<VEC> ld_words(const uint32_t* p) {
  Words<VEC> r;
  if constexpr (VEC == 4) {
    uint4 t = *reinterpret_cast<const uint4*>(p);
    r.w[0] = t.x; r.w[1] = t.y; r.w[2] = t.z; r.w[3] = t.w;
  } else if constexpr (VEC == 2) {
    uint2 t = *reinterpret_cast<const uint2*>(p);
    r.w[0] = t.x; r.w[1] = t.y;
  } else {
    r.w[0] = *p;
  }
  return r;
}

// Read-only path: frontier words of the level being expanded and the graph.
template <int VEC>
__device__ __forceinline__ Words<VEC> ldg_words(const uint32_t* p) {
  Words<VEC> r;
  if constexpr (VEC == 4) {
    uint4 t = __ldg(reinterpret_cast<const uint4*>(p));
    r.w[0] = t.x; r.w[1] = t.y; r.w[2] = t.z; r.w[3] = t.w;
  } else if constexpr (VEC == 2) {
    uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
    r.w[0] = t.x; r.w[1] = t.y;
  } else {
    r.w[0] = __ldg(p);
  }
  return r;
}

// Frontier-row gathers of the bottom-up step (random rows, L1 hit rate
// 14-21% on R-MAT 22). MSBFS_GATHER_LOAD picks the cache path: 0 the
// read-only path, 1 the same without allocating in L1, 2 L2 only. R-MAT
// scale 22, S=512, step ms: 7.54 / 8.03 / 7.63 -- the hubs' rows that L1
// keeps are worth its allocation traffic.
#ifndef MSBFS_GATHER_LOAD
#define MSBFS_GATHER_LOAD 0
#endif
template <int VEC>
__device__ __forceinline__ Words<VEC> gather_words(const uint32_t* p) {
  if constexpr (MSBFS_GATHER_LOAD == 1 && VEC == 4) {
    Words<VEC> r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3])
                 : "l"(p));
    return r;
  } else if constexpr (MSBFS_GATHER_LOAD == 2) {
    Words<VEC> r;
    if constexpr (VEC == 4) {
      uint4 t = __ldcg(reinterpret_cast<const uint4*>(p));
      r.w[0] = t.x; r.w[1] = t.y; r.w[2] = t.z; r.w[3] = t.w;
    } else if constexpr (VEC == 2) {
      uint2 t = __ldcg(reinterpret_cast<const uint2*>(p));
      r.w[0] = t.x; r.w[1] = t.y;
    } else {
      r.w[0] = __ldcg(p);
    }
    return r;
  } else {
    return ldg_words<VEC>(p);
  }
}

// L2-coherent read of words other blocks update with atomics this level.
template <int VEC>
__device__ __forceinline__ Words<VEC> ldcg_words(const uint32_t* p) {
  Words<VEC> r;
  if constexpr (VEC == 4) {
    uint4 t = __ldcg(reinterpret_cast<const uint4*>(p));
    r.w[0] = t.x; r.w[1] = t.y; r.w[2] = t.z; r.w[3] = t.w;
  } else if constexpr (VEC == 2) {
    uint2 t = __ldcg(reinterpret_cast<const uint2*>(p));
    r.w[0] = t.x; r.w[1] = t.y;
  } else {
    r.w[0] = __ldcg(p);
  }
  return r;
}

template <int VEC>
__device__ __forceinline__ void st_words(uint32_t* p, const Words<VEC>& r) {
  if constexpr (VEC == 4) {
    *reinterpret_cast<uint4*>(p) = make_uint4(r.w[0], r.w[1], r.w[2], r.w[3]);
  } else if constexpr (VEC == 2) {
    *reinterpret_cast<uint2*>(p) = make_uint2(r.w[0], r.w[1]);
  } else {
    *p = r.w[0];
  }
}

template <int VEC>
__device__ __forceinline__ bool any_bits(const Words<VEC>& a) {
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < VEC; ++j) x |= a.w[j];
  return x != 0;
}

__device__ __forceinline__ uint32_t nseg_of(uint32_t deg, uint32_t seg) {
  return deg ? (deg + seg - 1) / seg : 1u;
}

struct BlockQueue {
  uint32_t items[BQ_CAP];
  uint32_t count;
  uint32_t base;
  uint32_t warp_sum[LEVEL_BLOCK / 32];
  unsigned long long warp_edges[LEVEL_BLOCK / 32];
};

// Enqueue straight into the global queue (sources, and blocks whose staging
// area is full). Entry i of vertex v covers out-edges [i*seg, (i+1)*seg).
__device__ void enqueue_global(const LevelParams& p, uint32_t slot, uint32_t v, uint32_t seg) {
  const uint32_t deg = p.out_off[v + 1] - p.out_off[v];
  const uint32_t n = nseg_of(deg, seg);
  const uint32_t base = atomicAdd(&p.ctl->qcount[slot], n);
  atomicAdd(&p.ctl->qverts[slot], 1u);
  atomicAdd(&p.ctl->qedges[slot], (unsigned long long)deg);
  for (uint32_t i = 0; i < n; ++i)
    if (BCHECK(base + i < (slot == 0 ? p.qcap0 : p.qcap), CK_QUEUE_CAP))
      p.Q[slot][base + i] = ((unsigned long long)i << 32) | v;
}

__device__ __forceinline__ void bq_push(const LevelParams& p, BlockQueue& bq, uint32_t slot,
                                        uint32_t v) {
  const uint32_t pos = atomicAdd(&bq.count, 1u);
  if (pos < BQ_CAP)
    bq.items[pos] = v;
  else
    enqueue_global(p, slot, v, p.seg);
}

// Compacts the block's staged vertices into the global queue with one
// atomicAdd per block: per-item segment counts, block-wide exclusive scan.
__device__ void flush_block_queue(const LevelParams& p, BlockQueue& bq, uint32_t slot) {
  __syncthreads();
  const uint32_t n = min(bq.count, (uint32_t)BQ_CAP);
  if (n == 0) return;  // uniform: read after the barrier
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = (n + LEVEL_BLOCK - 1) / LEVEL_BLOCK;
  const uint32_t b = min(n, tid * per), e = min(n, b + per);
  uint32_t mine = 0;
  unsigned long long edges = 0;
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t v = bq.items[i];
    const uint32_t deg = p.out_off[v + 1] - p.out_off[v];
    mine += nseg_of(deg, p.seg);
    edges += deg;
  }
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(FULL, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  unsigned long long esum = edges;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(FULL, esum, o);
  if (lane == 31) bq.warp_sum[warp] = incl;
  if (lane == 0) bq.warp_edges[warp] = esum;
  __syncthreads();
  if (tid == 0) {
    uint32_t run = 0;
    unsigned long long etot = 0;
    for (int w = 0; w < LEVEL_BLOCK / 32; ++w) {
      uint32_t t = bq.warp_sum[w];
      bq.warp_sum[w] = run;
      run += t;
      etot += bq.warp_edges[w];
    }
    bq.base = atomicAdd(&p.ctl->qcount[slot], run);
    atomicAdd(&p.ctl->qverts[slot], n);
    atomicAdd(&p.ctl->qedges[slot], etot);
  }
  __syncthreads();
  uint32_t pos = bq.base + bq.warp_sum[warp] + incl - mine;
  unsigned long long* Q = p.Q[slot];
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t v = bq.items[i];
    const uint32_t deg = p.out_off[v + 1] - p.out_off[v];
    const uint32_t ns = nseg_of(deg, p.seg);
    for (uint32_t s = 0; s < ns; ++s, ++pos)
      if (BCHECK(pos < (slot == 0 ? p.qcap0 : p.qcap), CK_QUEUE_CAP))
        Q[pos] = ((unsigned long long)s << 32) | v;
  }
}

// Records distance d for the `newly` lanes of words [k0, k0+VEC) of vertex v.
// Bottom-up steps own their vertex (plain read-modify-write); top-down steps
// race with other blocks on the same words (atomicOr; the lanes are disjoint).
template <int VEC, bool ATOMIC>
__device__ __forceinline__ void record_level(const LevelParams& p, uint32_t v, uint32_t k0,
                                             const Words<VEC>& newly, uint32_t d) {
  const size_t VW = (size_t)p.V * p.W;
  const size_t off = (size_t)v * p.W + k0;
  if (d < (1u << p.NP)) {
    for (uint32_t b = 0; b < p.NP; ++b) {
      if (!((d >> b) & 1u)) continue;
      uint32_t* pb = p.planes + b * VW + off;
      if constexpr (ATOMIC) {
#pragma unroll
        for (int j = 0; j < VEC; ++j)
          if (newly.w[j]) atomicOr(pb + j, newly.w[j]);
      } else {
        Words<VEC> x = ld_words<VEC>(pb);
#pragma unroll
        for (int j = 0; j < VEC; ++j) x.w[j] |= newly.w[j];
        st_words<VEC>(pb, x);
      }
    }
  } else {
    // Deeper than the planes can encode: mark the lanes and write the rows.
    // With per-source reductions instead of rows, the deep lanes are folded
    // into the reductions here.
    uint32_t* dist = p.desc->dist;  // null when reductions or reachability are wanted
    SourceStats* st = p.desc->stats;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      uint32_t bits = newly.w[j];
      if (!bits) continue;
      atomicOr(p.ovf + off + j, bits);
      while ((dist || st) && bits) {
        const uint32_t t = __ffs(bits) - 1;
        bits &= bits - 1;
        const size_t s = (size_t)(k0 + j) * 32 + t;
        if (dist) {
          dist[s * p.V + v] = d;
        } else {
          atomicAdd(&st[s].sum, (unsigned long long)d);
          atomicMax(&st[s].ecc, d);
          atomicAdd(&st[s].reached, 1u);
        }
      }
    }
  }
}

// Per-thread work counts of one level (32-bit: a thread's share of a level
// stays far below 2^32; they are widened when the block reduces them).
struct LevelCounters {
  uint32_t active = 0, edges = 0, newv = 0, pairs = 0, rows = 0;
};

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t lane_word_mask(uint32_t P, uint32_t k) {
  const uint32_t lo = k * 32;
  if (P <= lo) return 0;
  const uint32_t rem = P - lo;
  return rem >= 32 ? FULL : ((1u << rem) - 1);
}

// Lane bits of the words [k0, k0+VEC) that are still worth discovering at
// level L (sources of this pass whose frontier is non-empty), from the
// block's shared copy (kept out of registers: the gather loops need them).
template <int VEC>
__device__ __forceinline__ Words<VEC> alive_lanes(const uint32_t* s_alive, uint32_t k0) {
  Words<VEC> m;
#pragma unroll
  for (int j = 0; j < VEC; ++j) m.w[j] = s_alive[k0 + j];
  return m;
}

// Visited/frontier/level/queue writes for a vertex owned by the calling group
// (all LPV lanes call it with their own VEC words).
// The visited words are read again here rather than held in registers
// through the gather loop (the group owns the vertex: nothing else writes
// them during the level).
template <int W, int VEC>
__device__ __forceinline__ void pull_commit(const LevelParams& p, BlockQueue& bq, uint32_t* s_lanes,
                                            uint32_t L, uint32_t v, uint32_t k0, uint32_t lig,
                                            const Words<VEC>& newly, LevelCounters& cnt) {
#pragma unroll
  for (int q = 0; q < VEC; ++q) {
    cnt.pairs += __popc(newly.w[q]);
    if (newly.w[q]) atomicOr(s_lanes + k0 + q, newly.w[q]);
  }
  // A lane whose words gained nothing leaves them as they are: its visited
  // words are unchanged, its frontier words of level L+1 are already zero
  // (cleared at level L-1) and its level-plane words need no bit. Late
  // levels discover a lane or two per vertex, so most pieces skip.
  if (any_bits<VEC>(newly)) {
    uint32_t* Fout = p.F[(L + 1) % 3];
    Words<VEC> nv = ld_words<VEC>(p.vis + (size_t)v * W + k0);
#pragma unroll
    for (int q = 0; q < VEC; ++q) nv.w[q] |= newly.w[q];
    st_words<VEC>(p.vis + (size_t)v * W + k0, nv);
    st_words<VEC>(Fout + (size_t)v * W + k0, newly);
    record_level<VEC, false>(p, v, k0, newly, L + 1);
  }
  if (lig == 0) {
    cnt.newv += 1;
    atomicOr(p.fbits[(L + 1) % 3] + (v >> 5), 1u << (v & 31));
    bq_push(p, bq, (L + 1) % 3, v);
  }
}

// With a sparse frontier, checking the 1-bit membership map first avoids most
// 16-byte row loads; with a dense one the extra dependent load costs more
// than it saves, so the controller turns the check off (`fb` null).
__device__ __forceinline__ bool in_frontier(const uint32_t* fb, uint32_t u) {
  return !fb || ((__ldg(fb + (u >> 5)) >> (u & 31)) & 1u);
}

// Vertex tiles a warp claims per cursor bump: small batches even out the end
// of a level (R-MAT scale 22, S=512, 8 blocks per SM, slices of 512: a step
// takes 8.59 ms with 2 tiles, 8.52 with 1, 8.83 with 4; at 6 blocks and
// slices of 256, 4 tiles had been 8% and 8 tiles 6% below 16).
#ifndef MSBFS_TILE_BATCH
#define MSBFS_TILE_BATCH 2
#endif
constexpr uint32_t TILE_BATCH = MSBFS_TILE_BATCH;

// In-neighbour id as gathered: FULL when absent or, with a frontier bitmap,
// outside the frontier (so its row is not loaded). The lane holding an id
// tests it once for its whole group before the id is shuffled out.
__device__ __forceinline__ uint32_t gather_id(const LevelParams& p, const uint32_t* fb,
                                              uint32_t u) {
  if (u != FULL && !BCHECK(u < p.V, CK_GATHER_ID)) return FULL;
  return (u != FULL && in_frontier(fb, u)) ? u : FULL;
}

// Bottom-up step over all vertices, in two parts.
// (1) Sliced vertices (in-degree > split): each warp takes one slice of one
//     vertex's in-edges, ORs the in-neighbours' frontier rows (every group of
//     the warp takes CH of them per round), publishes the partial candidate
//     words with atomicOr, and the last slice to arrive commits the vertex.
// (2) Every other vertex: a group of LPV lanes owns it, each lane holding VEC
//     of its W words; in-neighbours are gathered CH at a time (CH independent
//     16-byte loads in flight per lane) and the scan stops once the candidate
//     words cover every lane still to be discovered. Vertices with in-degree
//     >= heavy are scanned by the whole warp.
template <int W>
__device__ void pull_phase(const LevelParams& p, BlockQueue& bq, uint32_t* s_lanes,
                           const uint32_t* s_alive, uint32_t L, LevelCounters& cnt) {
  using G = Geo<W>;
  constexpr int VEC = G::VEC, LPV = G::LPV, GPW = G::GPW;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lig = lane % LPV;
  const uint32_t gbase = lane - lig;
  const uint32_t gid = lane / LPV;
  const uint32_t gmask = (LPV == 32) ? FULL : (((1u << LPV) - 1u) << gbase);
  const uint32_t k0 = lig * VEC;
  const uint32_t* __restrict__ Fin = p.F[L % 3];
  const uint32_t* __restrict__ fb =
      *(volatile uint32_t*)&p.ctl->use_bits ? p.fbits[L % 3] : nullptr;
  const uint32_t* __restrict__ in_off = p.in_off;
  const uint32_t* __restrict__ in_idx = p.in_idx;
  const uint32_t warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;

  // ---- (1) sliced high in-degree vertices. A warp takes its slices 32 at a
  // time and first tests their bits in p.hlive, so slices whose vertex needs
  // no lane any more (cleared below, for the rest of the pass) cost one bit
  // test instead of a chain of dependent loads.
  for (uint32_t cb = warp_g; cb < p.n_hchunks; cb += 32 * nwarps) {
    const uint32_t mine = cb + lane * nwarps;
    const bool live = mine < p.n_hchunks && ((p.hlive[mine >> 5] >> (mine & 31)) & 1u);
    uint32_t todo = __ballot_sync(FULL, live);
   while (todo) {
    const uint32_t ci = cb + (__ffs(todo) - 1) * nwarps;
    todo &= todo - 1;
    const HeavyChunk hk = p.hchunks[ci];
    const uint32_t v = hk.v;
    if (!BCHECK(v < p.V && hk.j < hk.nch, CK_SLICE)) continue;
    const uint32_t vb = __ldg(in_off + v);
    const uint32_t beg = vb + hk.j * p.split;
    const uint32_t end = min(__ldg(in_off + v + 1), beg + p.split);
    const Words<VEC> visw = ld_words<VEC>(p.vis + (size_t)v * W + k0);
    Words<VEC> needed, hc, shared_c;
    bool sat = true;
    uint32_t* hrow = p.hcand + (size_t)hk.h * W + k0;
    shared_c = ldcg_words<VEC>(hrow);
    const Words<VEC> lmask = alive_lanes<VEC>(s_alive, k0);
#pragma unroll
    for (int q = 0; q < VEC; ++q) {
      needed.w[q] = ~visw.w[q] & lmask.w[q];
      hc.w[q] = 0;
      sat &= (shared_c.w[q] & needed.w[q]) == needed.w[q];
    }
    // Every slice of v sees the same `needed` (only the committing slice
    // writes v's visited row, after all slices arrived).
    if (!__any_sync(FULL, any_bits<VEC>(needed))) {
      if (lane == 0) atomicAnd(&p.hlive[ci >> 5], ~(1u << (ci & 31)));
      continue;
    }
    if (hk.j == 0 && lane == 0) cnt.active += 1;
    if (!__all_sync(FULL, sat)) {
      // Each round the warp gathers GPW*CH in-neighbours; the ids of the next
      // round are fetched while this round's frontier rows are in flight, so
      // a round costs one memory latency, not two.
      constexpr int NI = LPV >= CH ? 1 : CH;  // ids held per lane
      uint32_t ids[NI];
#pragma unroll
      for (int j = 0; j < NI; ++j) {
        const uint32_t e = beg + gid * CH + (LPV >= CH ? lig : j);
        ids[j] = ((LPV < CH || lig < CH) && e < end) ? __ldg(in_idx + e) : FULL;
      }
      for (uint32_t base = beg; base < end; base += GPW * CH) {
        const uint32_t e0 = base + gid * CH;
        if (lig == 0 && e0 < end) cnt.edges += min((uint32_t)CH, end - e0);
        uint32_t u[CH];
        if constexpr (LPV >= CH) {
          const uint32_t mine = gather_id(p, fb, ids[0]);
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = __shfl_sync(FULL, mine, gbase + j);
        } else {
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = gather_id(p, fb, ids[j]);
        }
#pragma unroll
        for (int j = 0; j < NI; ++j) {
          const uint32_t e = e0 + GPW * CH + (LPV >= CH ? lig : j);
          ids[j] = ((LPV < CH || lig < CH) && e < end) ? __ldg(in_idx + e) : FULL;
        }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          if (u[j] != FULL) {
            cnt.rows += 1;
            Words<VEC> f = gather_words<VEC>(Fin + (size_t)u[j] * W + k0);
#pragma unroll
            for (int q = 0; q < VEC; ++q) hc.w[q] |= f.w[q];
          }
        }
        bool s2 = true;
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          uint32_t c = hc.w[q];
#pragma unroll
          for (int o = LPV; o < 32; o <<= 1) c |= __shfl_xor_sync(FULL, c, o);
          hc.w[q] = c;
          s2 &= (c & needed.w[q]) == needed.w[q];
        }
        if (__all_sync(FULL, s2)) break;
      }
      if (gid == 0) {
#pragma unroll
        for (int q = 0; q < VEC; ++q)
          if (hc.w[q] & needed.w[q]) atomicOr(hrow + q, hc.w[q] & needed.w[q]);
      }
    }
    __threadfence();
    uint32_t last = 0;
    if (lane == 0) last = (atomicAdd(p.hcount + hk.h, 1u) == hk.nch - 1) ? 1u : 0u;
    last = __shfl_sync(FULL, last, 0);
    if (last) {
      __threadfence();
      if (gid == 0) {
        const Words<VEC> fin = ldcg_words<VEC>(hrow);
        Words<VEC> newly, zero;
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          newly.w[q] = fin.w[q] & needed.w[q];
          zero.w[q] = 0;
        }
        st_words<VEC>(hrow, zero);
        const bool any_new = (__ballot_sync(gmask, any_bits<VEC>(newly)) & gmask) != 0;
        if (any_new) pull_commit<W, VEC>(p, bq, s_lanes, L, v, k0, lig, newly, cnt);
        if (lane == 0) p.hcount[hk.h] = 0;
      }
    }
   }
  }

  // ---- (2) all other vertices with in-edges, in the graph's work order
  // (ascending ids: neighbouring vertices share cache lines of the visited
  // and frontier rows), so vertices without in-edges cost nothing. Tiles are
  // claimed dynamically: work concentrates at some ids (R-MAT puts its hubs
  // first) and a static split would leave most warps idle behind a few.
  const uint32_t ntiles = (p.n_order + GPW - 1) / GPW;
  const uint32_t per_stripe = (ntiles + WORK_STRIPES - 1) / WORK_STRIPES;
  uint32_t stripe = warp_g % WORK_STRIPES, exhausted = 0;
  uint32_t tile = 0, tile_end = 0;
  [[maybe_unused]] uint32_t guard = 0;
  for (;;) {
    LOOP_GUARD(guard, ntiles + 2 * WORK_STRIPES + 2, CK_TILE_LOOP)
    if (tile == tile_end) {
      // Claim from the warp's stripe; move to the next once it runs dry.
      while (exhausted < WORK_STRIPES) {
        const uint32_t sb = stripe * per_stripe, se = min(sb + per_stripe, ntiles);
        uint32_t t0 = 0;
        if (lane == 0) t0 = sb < se ? sb + atomicAdd(&p.ctl->work[stripe][0], TILE_BATCH) : se;
        t0 = __shfl_sync(FULL, t0, 0);
        if (t0 < se) {
          tile = t0;
          tile_end = min(t0 + TILE_BATCH, se);
          break;
        }
        ++exhausted;
        stripe = (stripe + 1) % WORK_STRIPES;
      }
      if (tile == tile_end) break;  // every stripe is done
    }
    const uint32_t oi = tile * GPW + gid;
    ++tile;
    uint32_t v = 0, beg = 0, end = 0;
    if (oi < p.n_order) {
      const uint4 ent = __ldg(p.order + oi);
      if (BCHECK(ent.x < p.V && ent.y <= ent.z && ent.z <= p.E, CK_ORDER_ENTRY)) {
        v = ent.x;
        beg = ent.y;
        end = ent.z;
      }
    }
    Words<VEC> needed, cand;
#pragma unroll
    for (int j = 0; j < VEC; ++j) needed.w[j] = cand.w[j] = 0;
    if (end > beg) {
      const Words<VEC> visw = ld_words<VEC>(p.vis + (size_t)v * W + k0);
      const Words<VEC> lmask = alive_lanes<VEC>(s_alive, k0);
#pragma unroll
      for (int j = 0; j < VEC; ++j) needed.w[j] = ~visw.w[j] & lmask.w[j];
    }
    const bool need = (__ballot_sync(FULL, any_bits<VEC>(needed)) & gmask) != 0;
    const bool heavy = need && (end - beg) >= p.heavy;
    if (lig == 0 && need) cnt.active += 1;

    if (need && !heavy) {
      // The next chunk's in-neighbour ids are fetched while the current
      // chunk's frontier rows are in flight.
      constexpr int NI = LPV >= CH ? 1 : CH;  // ids held per lane
      uint32_t ids[NI];
      bool lane_sat = !any_bits<VEC>(needed);
#pragma unroll
      for (int j = 0; j < NI; ++j) {
        const uint32_t e = beg + (LPV >= CH ? lig : j);
        ids[j] = ((LPV < CH || lig < CH) && e < end) ? __ldg(in_idx + e) : FULL;
      }
      for (uint32_t e0 = beg; e0 < end; e0 += CH) {
        uint32_t u[CH];
        if constexpr (LPV >= CH) {
          const uint32_t mine = gather_id(p, fb, ids[0]);
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = __shfl_sync(gmask, mine, gbase + j);
        } else {
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = gather_id(p, fb, ids[j]);
        }
#pragma unroll
        for (int j = 0; j < NI; ++j) {
          const uint32_t e = e0 + CH + (LPV >= CH ? lig : j);
          ids[j] = ((LPV < CH || lig < CH) && e < end) ? __ldg(in_idx + e) : FULL;
        }
        Words<VEC> f[CH];
        if (lig == 0) cnt.edges += min((uint32_t)CH, end - e0);
        // A lane whose own words are covered skips its 16-byte pieces.
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          if (!lane_sat && u[j] != FULL) {
            cnt.rows += 1;
            f[j] = gather_words<VEC>(Fin + (size_t)u[j] * W + k0);
          } else {
#pragma unroll
            for (int q = 0; q < VEC; ++q) f[j].w[q] = 0;
          }
        }
        bool sat = true;
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          uint32_t c = cand.w[q];
#pragma unroll
          for (int j = 0; j < CH; ++j) c |= f[j].w[q];
          cand.w[q] = c;
          sat &= (c & needed.w[q]) == needed.w[q];
        }
        lane_sat = sat;
        if (__ballot_sync(gmask, !sat) == 0) break;
      }
    }

    uint32_t hmask = __ballot_sync(FULL, heavy && lig == 0);
    while (hmask) {
      const uint32_t hl = __ffs(hmask) - 1;
      hmask &= hmask - 1;
      const uint32_t hbeg = __shfl_sync(FULL, beg, hl);
      const uint32_t hend = __shfl_sync(FULL, end, hl);
      Words<VEC> hneed, hc;
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        hneed.w[q] = __shfl_sync(FULL, needed.w[q], hl + lig);
        hc.w[q] = 0;
      }
      constexpr int NI = LPV >= CH ? 1 : CH;  // ids held per lane (next round)
      uint32_t ids[NI];
#pragma unroll
      for (int j = 0; j < NI; ++j) {
        const uint32_t e = hbeg + gid * CH + (LPV >= CH ? lig : j);
        ids[j] = ((LPV < CH || lig < CH) && e < hend) ? __ldg(in_idx + e) : FULL;
      }
      for (uint32_t base = hbeg; base < hend; base += GPW * CH) {
        const uint32_t e0 = base + gid * CH;
        if (lig == 0 && e0 < hend) cnt.edges += min((uint32_t)CH, hend - e0);
        uint32_t u[CH];
        if constexpr (LPV >= CH) {
          const uint32_t mine = gather_id(p, fb, ids[0]);
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = __shfl_sync(FULL, mine, gbase + j);
        } else {
#pragma unroll
          for (int j = 0; j < CH; ++j) u[j] = gather_id(p, fb, ids[j]);
        }
#pragma unroll
        for (int j = 0; j < NI; ++j) {
          const uint32_t e = e0 + GPW * CH + (LPV >= CH ? lig : j);
          ids[j] = ((LPV < CH || lig < CH) && e < hend) ? __ldg(in_idx + e) : FULL;
        }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          if (u[j] != FULL) {
            cnt.rows += 1;
            Words<VEC> f = gather_words<VEC>(Fin + (size_t)u[j] * W + k0);
#pragma unroll
            for (int q = 0; q < VEC; ++q) hc.w[q] |= f.w[q];
          }
        }
        bool sat = true;
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          uint32_t c = hc.w[q];
#pragma unroll
          for (int o = LPV; o < 32; o <<= 1) c |= __shfl_xor_sync(FULL, c, o);
          hc.w[q] = c;
          sat &= (c & hneed.w[q]) == hneed.w[q];
        }
        if (__all_sync(FULL, sat)) break;
      }
      if (gbase == hl) cand = hc;
    }

    Words<VEC> newly;
#pragma unroll
    for (int q = 0; q < VEC; ++q) newly.w[q] = cand.w[q] & needed.w[q];
    const bool any_new = (__ballot_sync(FULL, any_bits<VEC>(newly)) & gmask) != 0;
    if (any_new) pull_commit<W, VEC>(p, bq, s_lanes, L, v, k0, lig, newly, cnt);
  }
}

// Top-down step over the frontier queue. A group takes one queue entry (a
// vertex and a slice of at most `seg` out-edges) and walks its edges; lanes
// that hit the same visited word in the same step (frequent when many
// frontier vertices share a hub) are merged into one atomicOr by the first
// of them, which then owns the follow-up writes for that word.
template <int W>
__device__ void push_phase(const LevelParams& p, BlockQueue& bq, uint32_t* s_lanes, uint32_t L,
                           LevelCounters& cnt) {
  using G = Geo<W>;
  constexpr int VEC = G::VEC, LPV = G::LPV, GPW = G::GPW;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lig = lane % LPV;
  const uint32_t gbase = lane - lig;
  const uint32_t gmask = (LPV == 32) ? FULL : (((1u << LPV) - 1u) << gbase);
  const uint32_t k0 = lig * VEC;
  const uint32_t d = L + 1;
  const uint32_t si = L % 3, so = (L + 1) % 3;
  // The sources' queue (level 0) uses shorter entries: a few hundred
  // sources would otherwise leave most groups idle behind long edge walks.
  const uint32_t seg = L == 0 ? p.seg0 : p.seg;
  const uint32_t* __restrict__ Fin = p.F[si];
  uint32_t* __restrict__ Fout = p.F[so];
  const unsigned long long* __restrict__ Qi = p.Q[si];
  const uint32_t nin = *(volatile uint32_t*)&p.ctl->qcount[si];
  const uint32_t group_g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GPW + lane / LPV;
  const uint32_t ngroups = ((gridDim.x * blockDim.x) >> 5) * GPW;

  for (uint32_t i = group_g; i < nin; i += ngroups) {
    const unsigned long long ent = Qi[i];
    const uint32_t u = (uint32_t)ent;
    const uint32_t sg = (uint32_t)(ent >> 32);
    if (!BCHECK(u < p.V, CK_PUSH_ENTRY)) continue;
    const Words<VEC> f = ldg_words<VEC>(Fin + (size_t)u * W + k0);
    const uint32_t ob = __ldg(p.out_off + u), oe = __ldg(p.out_off + u + 1);
    const uint32_t eb = ob + sg * seg;
    const uint32_t ee = min(oe, eb + seg);
    if (lig == 0) cnt.edges += ee - eb;
    // The next edge's target and its visited words are fetched while this
    // edge is processed. A stale visited word only widens `needed`; the
    // atomicOr's previous value decides what is new.
    uint32_t vn = eb < ee ? __ldg(p.out_idx + eb) : 0u;
    if (!BCHECK(vn < p.V, CK_PUSH_TARGET)) vn = 0;
    Words<VEC> vwn;
    if (eb < ee) vwn = ldcg_words<VEC>(p.vis + (size_t)vn * W + k0);
    for (uint32_t e = eb; e < ee; ++e) {
      const uint32_t v = vn;
      uint32_t* vrow = p.vis + (size_t)v * W + k0;
      const Words<VEC> vw = vwn;
      if (e + 1 < ee) {
        vn = __ldg(p.out_idx + e + 1);
        if (!BCHECK(vn < p.V, CK_PUSH_TARGET)) vn = 0;
        vwn = ldcg_words<VEC>(p.vis + (size_t)vn * W + k0);
      }
      bool found = false;
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        const uint32_t needed = f.w[q] & ~vw.w[q];
        if (needed) {
          const unsigned act = __activemask();
          const unsigned peers = __match_any_sync(act, (unsigned long long)(vrow + q));
          const uint32_t agg = __reduce_or_sync(peers, needed);
          const uint32_t leader = __ffs(peers) - 1;
          uint32_t prev = 0;
          if (lane == leader) prev = atomicOr(vrow + q, agg);
          prev = __shfl_sync(peers, prev, leader);
          const uint32_t nw = agg & ~prev;
          if (lane == leader && nw) {
            atomicOr(Fout + (size_t)v * W + k0 + q, nw);
            Words<1> one;
            one.w[0] = nw;
            record_level<1, true>(p, v, k0 + q, one, d);
            cnt.pairs += __popc(nw);
            atomicOr(s_lanes + k0 + q, nw);
            found = true;
          }
        }
      }
      if (__ballot_sync(gmask, found) != 0 && lane == gbase) {
        if (__ldcg(p.stamp + v) != d && atomicExch(p.stamp + v, d) != d) {
          atomicOr(p.fbits[so] + (v >> 5), 1u << (v & 31));
          bq_push(p, bq, so, v);
          cnt.newv += 1;
        }
      }
    }
  }
}

// Device-side level controller, run by the last block of each level.
__device__ void controller(const LevelParams& p, cudaGraphConditionalHandle h, uint32_t L,
                           uint32_t dir) {
  volatile LevelCtl* c = p.ctl;
  const uint32_t so = (L + 1) % 3;
  const uint32_t n_next = c->qverts[so];
  const unsigned long long m_next = c->qedges[so];
  if (L < LOG_CAP) {
    LevelRec r;
    r.level = L;
    r.dir = dir;
    r.frontier_vertices = c->qverts[L % 3];
    r.frontier_entries = c->qcount[L % 3];
    r.active = c->c_active;
    r.edges = c->c_edges;
    r.new_vertices = c->c_newv;
    r.new_pairs = c->c_pairs;
    r.rows = c->c_rows / (p.W >= 4 ? p.W / 4 : 1);  // counted per 16-byte piece
    r.t_start = c->t_start;
    r.t_end = globaltimer();
    p.log[L] = r;
  }
  c->c_active = 0;
  c->c_edges = 0;
  c->c_newv = 0;
  c->c_pairs = 0;
  c->c_rows = 0;
  c->t_start = ~0ull;
  if (dir == DIR_PUSH)
    c->push_levels = c->push_levels + 1;
  else
    c->pull_levels = c->pull_levels + 1;
  bool stop = false;
  if (n_next == 0) {
    stop = true;
  } else if (L + 1 >= p.max_levels) {
    c->status = c->status | STATUS_LEVEL_CAP;
    stop = true;
  }
  if (stop) {
    c->terminated = 1;
    if (h) cudaGraphSetConditional(h, 0);
    return;
  }
  const unsigned long long explored = c->explored + c->qedges[L % 3];
  c->explored = explored;
  uint32_t nd = dir;
  if (p.mode == MODE_PUSH) {
    nd = DIR_PUSH;
  } else if (p.mode == MODE_PULL) {
    nd = DIR_PULL;
  } else if (dir == DIR_PUSH) {
    // Go bottom-up once the frontier's out-edges exceed E / alpha. (Beamer's
    // unexplored-edge estimate does not apply: with many sources a vertex
    // sits in the frontier of several levels, so explored edges exceed E.)
    if (m_next * (unsigned long long)p.alpha > p.E) nd = DIR_PULL;
  } else {
    // Back to top-down once the frontier holds fewer than V / beta vertices.
    if ((unsigned long long)n_next * p.beta < p.V) nd = DIR_PUSH;
  }
  for (uint32_t k = 0; k < p.W; ++k) c->lanes[L & 1][k] = 0;  // becomes level L+2's collector
  const uint32_t sc = (L + 2) % 3;  // slot of level L-1, becomes level L+2
  c->qcount[sc] = 0;
  c->qverts[sc] = 0;
  c->qedges[sc] = 0;
  c->dir = nd;
  c->level = L + 1;
  c->done_blocks = 0;
  for (uint32_t k = 0; k < WORK_STRIPES; ++k) c->work[k][0] = 0;
  c->use_bits = (p.bits_div && (unsigned long long)n_next * p.bits_div < p.V) ? 1u : 0u;
  __threadfence();
  if (h) cudaGraphSetConditional(h, 1);
}

// Zeroes the frontier words of the n entries of queue slot `sl` (entries
// with a non-zero segment repeat a vertex, so only segment 0 clears).
template <int W>
__device__ __forceinline__ void clear_frontier_rows(const LevelParams& p, uint32_t sl, uint32_t n,
                                                    size_t t0, size_t nthreads) {
  const unsigned long long* Q = p.Q[sl];
  uint32_t* F = p.F[sl];
  const size_t total = (size_t)n * W;
  for (size_t i = t0; i < total; i += nthreads) {
    const unsigned long long ent = Q[i / W];
    if ((ent >> 32) == 0 && BCHECK((uint32_t)ent < p.V, CK_CLEAR_ENTRY))
      F[(size_t)(uint32_t)ent * W + i % W] = 0;
  }
}

// One level of the traversal, bottom-up (DIR_PULL) or top-down (DIR_PUSH):
// the two directions are separate kernels, each with its own register
// budget, and both sit in the level loop's body -- the pull kernel first --
// so the one whose direction the control block does not name returns at
// once. When a pull level's controller turns the traversal top-down, the
// push kernel of the same body iteration runs the next level. COUNT keeps
// the per-level work counters of the profiling log (the production form
// compiles them out; the discovered-pair count is always kept).
#ifndef MSBFS_PUSH_MIN_BLOCKS
#define MSBFS_PUSH_MIN_BLOCKS MSBFS_LEVEL_MIN_BLOCKS
#endif
template <int W, uint32_t DIR, bool COUNT>
__global__ void __launch_bounds__(LEVEL_BLOCK, DIR == DIR_PULL ? MSBFS_LEVEL_MIN_BLOCKS
                                                               : MSBFS_PUSH_MIN_BLOCKS)
    level_kernel(LevelParams p, cudaGraphConditionalHandle h) {
  __shared__ BlockQueue bq;
  __shared__ unsigned long long s_red[5][LEVEL_BLOCK / 32];
  __shared__ uint32_t s_lanes[W];
  __shared__ uint32_t s_alive[W];
  __shared__ uint32_t s_last;
  volatile LevelCtl* c = p.ctl;
  // Speculative launches of the host-driven loop, and the kernel of the
  // other direction in the loop body, return here.
  if (c->terminated || c->dir != DIR) return;
  const uint32_t L = c->level;
  if (threadIdx.x == 0) {
    bq.count = 0;
    atomicMin(&p.ctl->t_start, globaltimer());
  }
  if constexpr (DIR == DIR_PULL) {
    const uint32_t P = p.desc->num_sources;
    for (uint32_t k = threadIdx.x; k < W; k += blockDim.x)
      s_alive[k] = lane_word_mask(P, k) & c->lanes[L & 1][k];
  }
  for (uint32_t k = threadIdx.x; k < W; k += blockDim.x) s_lanes[k] = 0;
  __syncthreads();

  // Clear the frontier words of level L-1 (not read or written this level).
  {
    const uint32_t sc = (L + 2) % 3;
    clear_frontier_rows<W>(p, sc, c->qcount[sc], blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                           (size_t)gridDim.x * blockDim.x);
    uint32_t* fc = p.fbits[sc];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (p.V + 31) / 32;
         i += gridDim.x * blockDim.x)
      fc[i] = 0;
  }

  LevelCounters cnt;
  if constexpr (DIR == DIR_PULL)
    pull_phase<W>(p, bq, s_lanes, s_alive, L, cnt);
  else
    push_phase<W>(p, bq, s_lanes, L, cnt);
  flush_block_queue(p, bq, (L + 1) % 3);  // starts with a block barrier
  for (uint32_t k = threadIdx.x; k < W; k += blockDim.x)
    if (s_lanes[k]) atomicOr(&p.ctl->lanes[(L + 1) & 1][k], s_lanes[k]);

  unsigned long long vals[5] = {cnt.active, cnt.edges, cnt.newv, cnt.pairs, cnt.rows};
  if constexpr (!COUNT) vals[0] = vals[1] = vals[2] = vals[4] = 0;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    if (!COUNT && i != 3) continue;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vals[i] += __shfl_xor_sync(FULL, vals[i], o);
    if ((threadIdx.x & 31) == 0) s_red[i][threadIdx.x >> 5] = vals[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; ++i) {
      if (!COUNT && i != 3) continue;
      for (int w = 0; w < LEVEL_BLOCK / 32; ++w) tot[i] += s_red[i][w];
    }
    if (tot[0]) atomicAdd(&p.ctl->c_active, tot[0]);
    if (tot[1]) atomicAdd(&p.ctl->c_edges, tot[1]);
    if (tot[2]) atomicAdd(&p.ctl->c_newv, tot[2]);
    if (tot[4]) atomicAdd(&p.ctl->c_rows, tot[4]);
    if (tot[3]) {
      atomicAdd(&p.ctl->c_pairs, tot[3]);
      atomicAdd(&p.ctl->pairs, tot[3]);
    }
    __threadfence();
    const uint32_t prev = atomicAdd(&p.ctl->done_blocks, 1u);
    s_last = (prev == gridDim.x - 1);
    if (s_last) {
      __threadfence();
      controller(p, h, L, DIR);
    }
  }
}

// Level-0 frontier: lane i of word i/32 at vertex sources[i]. Duplicate
// sources share a vertex and are merged by atomicOr; the vertex is enqueued
// once (stamp 0).
template <int W>
__global__ void init_kernel(LevelParams p) {
  const PassDesc* dsc = p.desc;
  const uint32_t P = dsc->num_sources;
  unsigned long long ok = 0;
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
    const uint32_t s = dsc->sources[i];
    if (s >= p.V) {
      atomicOr(&p.ctl->status, STATUS_BAD_SOURCE);
      continue;
    }
    const uint32_t bit = 1u << (i & 31);
    const size_t w = (size_t)s * W + (i >> 5);
    atomicOr(p.vis + w, bit);
    atomicOr(p.F[0] + w, bit);
    atomicOr(&p.ctl->lanes[0][i >> 5], bit);
    atomicOr(p.fbits[0] + (s >> 5), 1u << (s & 31));
    if (atomicExch(p.stamp + s, 0u) != 0u) enqueue_global(p, 0, s, p.seg0);
    ++ok;
  }
  if (ok) atomicAdd(&p.ctl->pairs, ok);
  if (threadIdx.x == 0) {
    p.ctl->dir = (p.mode == MODE_PULL) ? DIR_PULL : DIR_PUSH;
    p.ctl->t_start = ~0ull;
  }
}

__device__ __forceinline__ uint32_t bit_length(uint32_t x) { return x ? 32 - __clz(x) : 0; }

// Materialisation. A block stages a tile of the visited words and level
// planes in shared memory, one coalesced 16-byte load per thread per array
// (MAT_TILE_WORDS words, 4 KB), transposed to [word][vertex] so that a warp
// reads one word of 64 consecutive vertices without bank conflicts. Each of
// the 16 (word, 64-vertex segment) columns of a tile then gives 32 distance
// rows, written as 256-byte segments (one 8-byte store per lane per row).
// Staging keeps every global load coalesced; the earlier form, where each
// lane loaded one 4-byte word per vertex (64-byte stride) and relied on the
// warps sharing a tile to meet in L1, ran 3.9 to 5.6 ms on R-MAT scale 22,
// S=512 depending on how closely those warps kept in step.
constexpr int MAT_TILE_WORDS = MAT_BLOCK * 4;
constexpr int MAT_NPMAX = 8;
constexpr int MAT_COLS = 16;  // (word, 64-vertex segment) columns per tile
#ifndef MSBFS_MAT_MIN_BLOCKS
#define MSBFS_MAT_MIN_BLOCKS 5
#endif
constexpr int MAT_MIN_BLOCKS = MSBFS_MAT_MIN_BLOCKS;

template <int W>
struct MatGeo {
  static constexpr int TW = W <= 16 ? W : 16;     // words per vertex in a tile
  static constexpr int TV = MAT_TILE_WORDS / TW;  // vertices per tile
  // Shared row stride in words: even (8-byte column reads) and, for TW = 16,
  // conflict-free for the transposing stores (bank = 8q + 2k + vertex).
  static constexpr int RS = TV + 2;
  static constexpr int ARR = TW * RS;             // shared words per array
  static_assert(TW * (TV / 64) == MAT_COLS, "16 columns per tile");
};

// Output side of a pass, read from the descriptor once per thread.
struct MatOut {
  uint32_t* dist;
  uint32_t* reach;
  uint32_t reach_wpv, reach_col;
  uint8_t* dist8;  // non-null: rows as one byte per distance (all below 255)
};

// Byte transpose of four words: byte i of r[m] is byte m of a[i].
__device__ __forceinline__ void byte_transpose4(uint32_t a0, uint32_t a1, uint32_t a2,
                                                uint32_t a3, uint32_t* r) {
  const uint32_t t0 = __byte_perm(a0, a1, 0x5140), t1 = __byte_perm(a0, a1, 0x7362);
  const uint32_t t2 = __byte_perm(a2, a3, 0x5140), t3 = __byte_perm(a2, a3, 0x7362);
  r[0] = __byte_perm(t0, t2, 0x5410);
  r[1] = __byte_perm(t0, t2, 0x7632);
  r[2] = __byte_perm(t1, t3, 0x5410);
  r[3] = __byte_perm(t1, t3, 0x7632);
}

// Transposes the 8x8 bit matrix held in (lo, hi), row r in byte r and column
// c in bit c of each byte, by three exchanges of 1x1, 2x2 and 4x4 blocks
// across the diagonal (Knuth's delta swaps); the 64-bit shifts by 7 and 14
// stay inside each 32-bit half, the one by 28 moves a nibble between them.
__device__ __forceinline__ void bit_transpose8(uint32_t& lo, uint32_t& hi) {
  uint32_t t;
  t = (lo ^ (lo >> 7)) & 0x00AA00AAu;
  lo ^= t ^ (t << 7);
  t = (hi ^ (hi >> 7)) & 0x00AA00AAu;
  hi ^= t ^ (t << 7);
  t = (lo ^ (lo >> 14)) & 0x0000CCCCu;
  lo ^= t ^ (t << 14);
  t = (hi ^ (hi >> 14)) & 0x0000CCCCu;
  hi ^= t ^ (t << 14);
  t = (lo ^ (hi << 4)) & 0xF0F0F0F0u;
  lo ^= t;
  hi ^= t >> 4;
}

// The distances of one vertex to the 32 sources of a word, as bytes: q[k]
// byte i is source 4k+i's distance, 0xFF where the visited word xs has no
// bit. pl[b] bit j is bit b of source j's distance; unreached sources get
// every plane bit set. Planes 0-3 and 4-7 are byte-transposed, so that word m
// of each pair holds byte m (sources 8m..8m+7) of all eight planes, and an
// 8x8 bit transpose of that pair turns plane-major bits into one byte per
// source.
template <int NPU>
__device__ __forceinline__ void pack_distances(uint32_t xs, const uint32_t* pl, uint32_t* q) {
  uint32_t pb[8];
#pragma unroll
  for (int b = 0; b < 8; ++b) pb[b] = (b < NPU ? pl[b < NPU ? b : 0] : 0u) | ~xs;
  uint32_t lo[4], hi[4];
  byte_transpose4(pb[0], pb[1], pb[2], pb[3], lo);
  byte_transpose4(pb[4], pb[5], pb[6], pb[7], hi);
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    bit_transpose8(lo[m], hi[m]);
    q[2 * m] = lo[m];
    q[2 * m + 1] = hi[m];
  }
}

// Byte i of w as a u32 distance, 0xFF (unreached) widened to DIST_MAX. With
// at most 7 planes every reached distance is below 128, so one byte permute
// that replicates the byte's sign bit does both (prmt selector nibbles with
// bit 3 set copy the sign); with 8 planes the unreached byte is compared.
template <int NPU>
__device__ __forceinline__ uint32_t widen_distance(uint32_t w, uint32_t i) {
  if constexpr (NPU <= 7) {
    const uint32_t sel = i | ((i | 8u) << 4) | ((i | 8u) << 8) | ((i | 8u) << 12);
    uint32_t d;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(w), "r"(sel));
    return d;
  } else {
    const uint32_t d = (w >> (8 * i)) & 0xFFu;
    return d == 0xFFu ? DIST_MAX : d;
  }
}

// Writes the rows of column cs of the staged tile: word cw = g*TW + c of the
// 64 vertices from v0 + 64*seg, i.e. sources 32cw .. 32cw+31 of the pass.
// Lane l owns vertices 2l and 2l+1 of the segment. NPU (planes in use) is a
// template argument so the plane words stay in registers. Lanes flagged in
// ovf (deeper than the planes encode) were written by the level kernel and
// are skipped. `packed` (no ovf lane, every distance below 255) takes the
// transposed form: each vertex's 32 distances are computed at once as bytes
// and a row costs one byte select per vertex, against one bit extraction
// per plane per source in the per-bit form.
template <int W, int NPU>
__device__ __forceinline__ void mat_column(const LevelParams& p, const MatOut& out,
                                           const uint32_t* sh, uint32_t v0, uint32_t g,
                                           uint32_t cs, uint32_t lane, uint32_t P, bool use_ovf,
                                           bool packed, bool vec_ok) {
  using G = MatGeo<W>;
  const uint32_t V = p.V;
  const uint32_t c = cs % G::TW;
  const uint32_t seg = cs / G::TW;
  const uint32_t cw = g * G::TW + c;
  const uint32_t vloc = seg * 64 + 2 * lane;
  const uint32_t vl = v0 + vloc;
  uint32_t xs[2], ov[2] = {0, 0};
  uint32_t pl[NPU > 0 ? NPU : 1][2];
  {
    const uint2 t = *reinterpret_cast<const uint2*>(sh + c * G::RS + vloc);
    xs[0] = t.x;
    xs[1] = t.y;
  }
#pragma unroll
  for (int b = 0; b < NPU; ++b) {
    const uint2 t = *reinterpret_cast<const uint2*>(sh + (1 + b) * G::ARR + c * G::RS + vloc);
    pl[b][0] = t.x;
    pl[b][1] = t.y;
  }
  if (use_ovf) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (vl + t < V) {
        uint32_t* a = p.ovf + (size_t)(vl + t) * W + cw;
        ov[t] = *a;
        if (ov[t]) *a = 0;
      }
    }
  }
  if (out.reach) {
#pragma unroll
    for (int t = 0; t < 2; ++t)
      if (vl + t < V) out.reach[(size_t)(vl + t) * out.reach_wpv + out.reach_col + cw] = xs[t];
    return;
  }
  const uint32_t s0 = cw * 32;
  const uint32_t jn = min(32u, P - s0);
  if (packed) {
    uint32_t q[2][8];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      uint32_t plt[NPU > 0 ? NPU : 1];
#pragma unroll
      for (int b = 0; b < NPU; ++b) plt[b] = pl[b][t];
      pack_distances<NPU>(xs[t], plt, q[t]);
    }
    const bool full = vec_ok && vl + 1 < V;
    if (out.dist8) {
      uint8_t* row = out.dist8 + (size_t)s0 * V + vl;
#pragma unroll
      for (uint32_t j = 0; j < 32; ++j, row += V) {
        if (j >= jn) break;
        const uint32_t i = j & 3;
        const uint32_t two = __byte_perm(q[0][j >> 2], q[1][j >> 2], i | ((4 + i) << 4));
        if (full) {
          *reinterpret_cast<uint16_t*>(row) = (uint16_t)two;
        } else {
          if (vl < V) row[0] = (uint8_t)two;
          if (vl + 1 < V) row[1] = (uint8_t)(two >> 8);
        }
      }
    } else {
      uint32_t* row = out.dist + (size_t)s0 * V + vl;
#pragma unroll
      for (uint32_t j = 0; j < 32; ++j, row += V) {
        if (j >= jn) break;
        const uint32_t d0 = widen_distance<NPU>(q[0][j >> 2], j & 3);
        const uint32_t d1 = widen_distance<NPU>(q[1][j >> 2], j & 3);
        if (full) {
          *reinterpret_cast<uint2*>(row) = make_uint2(d0, d1);
        } else {
          if (vl < V) row[0] = d0;
          if (vl + 1 < V) row[1] = d1;
        }
      }
    }
    return;
  }
  if (out.dist8) {
    // Byte rows: no lane is deeper than the planes here (every distance is
    // below 255), so there is no ovf lane to skip.
    for (uint32_t j = 0; j < jn; ++j) {
      uint8_t dv[2];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        uint32_t val = 0;
#pragma unroll
        for (int b = 0; b < NPU; ++b) val |= ((pl[b][t] >> j) & 1u) << b;
        dv[t] = ((xs[t] >> j) & 1u) ? (uint8_t)val : (uint8_t)0xFF;
      }
      uint8_t* row = out.dist8 + (size_t)(s0 + j) * V + vl;
      if (vec_ok && vl + 1 < V) {
        *reinterpret_cast<uchar2*>(row) = make_uchar2(dv[0], dv[1]);
      } else {
#pragma unroll
        for (int t = 0; t < 2; ++t)
          if (vl + t < V) row[t] = dv[t];
      }
    }
    return;
  }
  uint32_t* dist = out.dist;
  const bool any_ovf = (ov[0] | ov[1]) != 0;
  const bool full = vec_ok && vl + 1 < V;
  for (uint32_t j = 0; j < jn; ++j) {
    uint32_t dv[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      uint32_t val = 0;
#pragma unroll
      for (int b = 0; b < NPU; ++b) val |= ((pl[b][t] >> j) & 1u) << b;
      dv[t] = ((xs[t] >> j) & 1u) ? val : DIST_MAX;
    }
    uint32_t* row = dist + (size_t)(s0 + j) * V + vl;
    bool skip = false;
    if (any_ovf) skip = (((ov[0] & xs[0]) | (ov[1] & xs[1])) >> j) & 1u;
    if (full && !skip) {
      *reinterpret_cast<uint2*>(row) = make_uint2(dv[0], dv[1]);
    } else {
#pragma unroll
      for (int t = 0; t < 2; ++t)
        if (vl + t < V && !(((ov[t] & xs[t]) >> j) & 1u)) row[t] = dv[t];
    }
  }
}

// 32x32 bit-matrix transpose across a warp: lane j returns the word whose bit
// t is bit j of lane t's x (five exchange steps of halving width).
__device__ __forceinline__ uint32_t transpose32(uint32_t x, uint32_t lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const uint32_t m = s == 16  ? 0x0000FFFFu
                       : s == 8 ? 0x00FF00FFu
                       : s == 4 ? 0x0F0F0F0Fu
                       : s == 2 ? 0x33333333u
                                : 0x55555555u;
    const uint32_t y = __shfl_xor_sync(FULL, x, s);
    x = (lane & s) ? ((x & ~m) | ((y & ~m) >> s)) : ((x & m) | ((y & m) << s));
  }
  return x;
}

constexpr int RED_BLOCK = 256;
#ifndef MSBFS_RED_MIN_BLOCKS
// R-MAT scale 22, S=512: 3 blocks (80 registers, a few spills) 0.82 ms,
// 2 blocks (113 registers) 0.96 ms, 4 blocks (64 registers) 0.92 ms.
#define MSBFS_RED_MIN_BLOCKS 3
#endif
constexpr int RED_MIN_BLOCKS = MSBFS_RED_MIN_BLOCKS;
constexpr uint32_t RED_CHUNK = 2048;  // vertices per reduction work item

template <int VEC>
__device__ __forceinline__ bool any_word(const Words<VEC>& x) {
  uint32_t a = 0;
#pragma unroll
  for (int j = 0; j < VEC; ++j) a |= x.w[j];
  return a != 0;
}

// Per-source reductions (distance sum, reached count, eccentricity) straight
// from the visited words and level planes, with no S*V matrix. A warp item is
// one group of G = min(4, W) words of RED_CHUNK consecutive vertices; lane l
// loads the group of vertex vb + l as one vector (the next tile's visited
// group is fetched while this one is reduced). For each word c of the group
// the warp transposes the visited word and each level plane (32x32 bits), so
// lane j holds source 32c+j's bits over the 32 vertices: the reached count is
// a popcount, the distance sum a popcount per plane, the eccentricity the
// largest plane pattern present. Plane bits are a subset of visited bits, so
// tiles without a visited bit skip the plane loads, and only words read
// non-zero are written back as zero (the next pass starts from clean
// buffers). Lanes flagged in ovf (deeper than the planes encode) were folded
// in by the level kernel.
template <int W>
__global__ void __launch_bounds__(RED_BLOCK, RED_MIN_BLOCKS) reduce_kernel(LevelParams p) {
  constexpr int G = W >= 4 ? 4 : W;
  const PassDesc* dsc = p.desc;
  SourceStats* st = dsc->stats;
  if (!st) return;
  const uint32_t P = dsc->num_sources;
  const uint32_t Wu = (P + 31) / 32;
  const uint32_t ngroups = (Wu + G - 1) / G;
  const uint32_t dmax = p.ctl->level;
  const uint32_t npu = min(min(p.NP, bit_length(dmax)), (uint32_t)MAT_NPMAX);
  const bool use_ovf = dmax >= (1u << p.NP);
  const uint32_t lane = threadIdx.x & 31;
  const size_t VW = (size_t)p.V * W;
  const size_t nitems = (size_t)((p.V + RED_CHUNK - 1) / RED_CHUNK) * ngroups;
  const size_t warp_g = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  Words<G> zero;
#pragma unroll
  for (int j = 0; j < G; ++j) zero.w[j] = 0;
  for (size_t it = warp_g; it < nitems; it += nwarps) {
    const uint32_t g = (uint32_t)(it % ngroups);
    const uint32_t v0 = (uint32_t)(it / ngroups) * RED_CHUNK;
    const uint32_t v_end = min(v0 + RED_CHUNK, p.V);
    unsigned long long sum[G];
    uint32_t cnt[G], ecc[G];
#pragma unroll
    for (int i = 0; i < G; ++i) {
      sum[i] = 0;
      cnt[i] = ecc[i] = 0;
    }
    Words<G> xn = zero;
    if (v0 + lane < v_end) xn = ld_words<G>(p.vis + (size_t)(v0 + lane) * W + (size_t)g * G);
    for (uint32_t vb = v0; vb < v_end; vb += 32) {
      const uint32_t v = vb + lane;
      const size_t a = (size_t)v * W + (size_t)g * G;
      const Words<G> x = xn;
      xn = zero;
      if (v + 32 < v_end) xn = ld_words<G>(p.vis + a + 32 * (size_t)W);
      const bool any = any_word(x);
      if (__ballot_sync(FULL, any) == 0) continue;  // warp-uniform
      Words<G> o = zero, pl[MAT_NPMAX];
#pragma unroll
      for (int b = 0; b < MAT_NPMAX; ++b) pl[b] = zero;
      if (any) {
        st_words<G>(p.vis + a, zero);
        if (use_ovf) o = ld_words<G>(p.ovf + a);
#pragma unroll
        for (int b = 0; b < MAT_NPMAX; ++b)
          if (b < (int)npu) pl[b] = ld_words<G>(p.planes + b * VW + a);
        if (any_word(o)) st_words<G>(p.ovf + a, zero);
#pragma unroll
        for (int b = 0; b < MAT_NPMAX; ++b)
          if (b < (int)npu && any_word(pl[b])) st_words<G>(p.planes + b * VW + a, zero);
      }
#pragma unroll
      for (int i = 0; i < G; ++i) {
        if (__ballot_sync(FULL, x.w[i] != 0) == 0) continue;  // warp-uniform
        const uint32_t xv = x.w[i] & ~o.w[i];  // lanes with an in-plane distance
        const uint32_t X = transpose32(xv, lane);
        cnt[i] += __popc(X);
        uint32_t cand = X, e = 0;
#pragma unroll
        for (int b = MAT_NPMAX - 1; b >= 0; --b) {
          if (b >= (int)npu) continue;  // npu is warp-uniform
          const uint32_t Pt = transpose32(pl[b].w[i] & xv, lane);
          sum[i] += (unsigned long long)__popc(Pt) << b;
          const uint32_t hi = cand & Pt;
          if (hi) {
            cand = hi;
            e |= 1u << b;
          }
        }
        if (X) ecc[i] = max(ecc[i], e);
      }
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      const uint32_t s = 32 * (g * G + i) + lane;
      if (cnt[i] && s < P) {
        atomicAdd(&st[s].sum, sum[i]);
        atomicMax(&st[s].ecc, ecc[i]);
        atomicAdd(&st[s].reached, cnt[i]);
      }
    }
  }
}

// Stages arrays A0..A1 of one tile (array 0 is the visited words, array
// a > 0 plane a - 1): this thread's four words of each, transposed into
// shared memory ([word][vertex] per array), zeroing in global memory the
// words that were not zero when `clear` is set. All loads of the range are
// issued before the first shared store so that their latencies overlap.
template <int W, int A0, int A1>
__device__ __forceinline__ void stage_arrays(const LevelParams& p, uint32_t* sh, size_t gw,
                                             bool inb, bool vec_planes, bool clear, uint32_t o) {
  using G = MatGeo<W>;
  constexpr int N = A1 - A0 + 1;
  const size_t VW = (size_t)p.V * W;
  uint32_t x[N][4];
  bool vec[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const int a = A0 + i;
    const uint32_t* src = a == 0 ? p.vis : p.planes + (size_t)(a - 1) * VW;
    vec[i] = inb && (a == 0 || vec_planes);
#pragma unroll
    for (int k = 0; k < 4; ++k) x[i][k] = 0;
    if (vec[i]) {
      const uint4 t = *reinterpret_cast<const uint4*>(src + gw);
      x[i][0] = t.x;
      x[i][1] = t.y;
      x[i][2] = t.z;
      x[i][3] = t.w;
    } else if constexpr (W <= 16) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (gw + k < VW) x[i][k] = src[gw + k];
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const int a = A0 + i;
    uint32_t* src = a == 0 ? p.vis : p.planes + (size_t)(a - 1) * VW;
    if (clear) {
      if (vec[i]) {
        if (x[i][0] | x[i][1] | x[i][2] | x[i][3])
          *reinterpret_cast<uint4*>(src + gw) = make_uint4(0, 0, 0, 0);
      } else if constexpr (W <= 16) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (gw + k < VW && x[i][k]) src[gw + k] = 0;
      }
    }
    uint32_t* dst = sh + a * G::ARR;
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[((o + k) % G::TW) * G::RS + (o + k) / G::TW] = x[i][k];
  }
}

// Stages the visited words and the NPU planes in use of one tile, at most
// five arrays in flight at a time (the register budget of 5 blocks per SM).
template <int W, int NPU>
__device__ __forceinline__ void stage_tile(const LevelParams& p, uint32_t* sh, size_t gw,
                                           bool inb, bool vec_planes, bool clear, uint32_t o) {
  stage_arrays<W, 0, (NPU < 4 ? NPU : 4)>(p, sh, gw, inb, vec_planes, clear, o);
  if constexpr (NPU > 4) stage_arrays<W, 5, NPU>(p, sh, gw, inb, vec_planes, clear, o);
}

// Turns visited words + level planes into the source-major u32 distance rows
// (or copies the visited words out as a reachability bitmask) and zeroes the
// words it read, so the next pass starts from clean buffers. Blocks take
// (vertex tile, word group) items; see MatGeo for the tile. Passes that want
// per-source reductions run reduce_kernel instead.
template <int W>
__global__ void __launch_bounds__(MAT_BLOCK, MAT_MIN_BLOCKS)
    materialize_kernel(LevelParams p, uint32_t phase) {
  using G = MatGeo<W>;
  extern __shared__ uint32_t mat_sh[];  // [1 + NP][TW][RS]: visited words, then planes
  const PassDesc* dsc = p.desc;
  if (dsc->stats) return;
  const uint32_t P = dsc->num_sources;
  const uint32_t Wu = (P + 31) / 32;
  const uint32_t dmax = p.ctl->level;
  const uint32_t npu = min(min(p.NP, bit_length(dmax)), (uint32_t)MAT_NPMAX);
  const bool use_ovf = dmax >= (1u << p.NP);
  // Every reached distance fits the planes and stays below the 0xFF marker.
  const bool packed = !use_ovf && dmax < 255u;
  // Byte rows when the pass asks for them and every distance fits a byte
  // (0xFF is kept for unreachable); the control block tells the host.
  const bool narrow = dsc->dist8 && !dsc->reach && dmax < 255u;
  if (phase == MAT_BYTES && !narrow) return;
  // Word columns this launch writes, whether as bytes, and whether it
  // clears the state it read (the last launch over the pass does).
  const uint32_t wsplit = min(dsc->row_split / 32, Wu);
  const uint32_t wlo = phase == MAT_BYTES ? wsplit : 0u;
  const uint32_t whi = (phase == MAT_WIDE && narrow) ? wsplit : Wu;
  const bool bytes = phase == MAT_BYTES || (phase == MAT_ALL && narrow);
  const bool clear = phase != MAT_BYTES;
  if (bytes && blockIdx.x == 0 && threadIdx.x == 0) p.ctl->narrow = 1;
  const MatOut out{dsc->dist, dsc->reach, dsc->reach_wpv, dsc->reach_col,
                   bytes ? dsc->dist8 : nullptr};
  const uint32_t V = p.V;
  const size_t VW = (size_t)V * W;
  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31;
  const uint32_t warp = tid >> 5;
  const bool vec_ok = bytes ? (V % 2 == 0) && (((uintptr_t)out.dist8 & 1) == 0)
                            : (V % 2 == 0) && (((uintptr_t)out.dist & 7) == 0);
  const uint32_t ngu = (Wu + G::TW - 1) / G::TW;  // word groups in use
  const size_t nitems = (size_t)((V + G::TV - 1) / G::TV) * ngu;
  const uint32_t o = 4 * tid;  // tile word offset of this thread's four words
  // Plane b starts b*V*W words into the planes buffer: 16-byte aligned only
  // when V*W is a multiple of 4 (always for W >= 4).
  const bool vec_planes = VW % 4 == 0;
  for (size_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const uint32_t g = (uint32_t)(it % ngu);
    const uint32_t v0 = (uint32_t)(it / ngu) * G::TV;
    // Global word index of this thread's four words: the tile is contiguous
    // when a vertex's words fit in one group (W <= 16); otherwise it is 64
    // runs of 16 words.
    size_t gw;
    bool inb;
    if constexpr (W <= 16) {
      gw = (size_t)v0 * W + o;
      inb = gw + 3 < VW;
    } else {
      gw = (size_t)(v0 + o / 16) * W + 16 * g + (o % 16);
      inb = v0 + o / 16 < V;
    }
    switch (npu) {
#define STAGE_CASE(n) \
  case n: stage_tile<W, n>(p, mat_sh, gw, inb, vec_planes, clear, o); break;
      STAGE_CASE(0) STAGE_CASE(1) STAGE_CASE(2) STAGE_CASE(3) STAGE_CASE(4)
      STAGE_CASE(5) STAGE_CASE(6) STAGE_CASE(7) STAGE_CASE(8)
#undef STAGE_CASE
      default: break;
    }
    __syncthreads();
    for (uint32_t cs = warp; cs < MAT_COLS; cs += MAT_BLOCK / 32) {
      const uint32_t cw = g * G::TW + cs % G::TW;
      if (cw < wlo || cw >= whi) continue;  // no sources of this launch in this word
      switch (npu) {
#define MAT_CASE(n) \
  case n: mat_column<W, n>(p, out, mat_sh, v0, g, cs, lane, P, use_ovf, packed, vec_ok); break;
        MAT_CASE(0) MAT_CASE(1) MAT_CASE(2) MAT_CASE(3) MAT_CASE(4)
        MAT_CASE(5) MAT_CASE(6) MAT_CASE(7) MAT_CASE(8)
#undef MAT_CASE
        default: break;
      }
    }
    __syncthreads();
  }
}

size_t materialize_items(uint32_t V, uint32_t W) {
  const uint32_t tw = W <= 16 ? W : 16;
  const uint32_t tv = MAT_TILE_WORDS / tw;
  return (size_t)((V + tv - 1) / tv) * ((W + tw - 1) / tw);
}

size_t materialize_smem_bytes(uint32_t W, uint32_t NP) {
  const uint32_t tw = W <= 16 ? W : 16;
  const uint32_t tv = MAT_TILE_WORDS / tw;
  const uint32_t np = NP < (uint32_t)MAT_NPMAX ? NP : (uint32_t)MAT_NPMAX;
  return (size_t)(1 + np) * tw * (tv + 2) * sizeof(uint32_t);
}

// Zeroes the frontier rows left after the loop has stopped: those of the
// last expanded level L and, when the level cap stopped a traversal that was
// still going, those of level L + 1 (empty after a normal stop).
template <int W>
__global__ void cleanup_kernel(LevelParams p) {
  const uint32_t L = p.ctl->level;
  for (uint32_t k = 0; k < 2; ++k)
    clear_frontier_rows<W>(p, (L + k) % 3, p.ctl->qcount[(L + k) % 3],
                           blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                           (size_t)gridDim.x * blockDim.x);
}

// Traversed edges of a distance matrix (crates/cli/src/bench.rs:478-491).
__global__ void traversed_edges_kernel(uint32_t V, const uint32_t* __restrict__ off,
                                       const uint32_t* __restrict__ dist, uint32_t S,
                                       unsigned long long* out) {
  unsigned long long acc = 0;
  const size_t total = (size_t)S * V;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    if (dist[i] != DIST_MAX) {
      const uint32_t v = (uint32_t)(i % V);
      acc += __ldg(off + v + 1) - __ldg(off + v);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// ------------------------------------------------------------------ host side

template <int W>
static void fill_info(int num_sms, uint32_t NP, LevelKernelInfo* k) {
  k->init = (void*)init_kernel<W>;
  k->level[DIR_PUSH][0] = (void*)level_kernel<W, DIR_PUSH, false>;
  k->level[DIR_PUSH][1] = (void*)level_kernel<W, DIR_PUSH, true>;
  k->level[DIR_PULL][0] = (void*)level_kernel<W, DIR_PULL, false>;
  k->level[DIR_PULL][1] = (void*)level_kernel<W, DIR_PULL, true>;
  k->materialize = (void*)materialize_kernel<W>;
  k->reduce = (void*)reduce_kernel<W>;
  k->cleanup = (void*)cleanup_kernel<W>;
  k->level_block = LEVEL_BLOCK;
  // The counting form runs at the production form's grid (it is only run
  // for its counters; the roofline's durations come from the production form).
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, level_kernel<W, DIR_PULL, false>,
                                                LEVEL_BLOCK, 0);
  k->level_grids[DIR_PULL] = num_sms * (occ < 1 ? 1 : occ);
  occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, level_kernel<W, DIR_PUSH, false>,
                                                LEVEL_BLOCK, 0);
  k->level_grids[DIR_PUSH] = num_sms * (occ < 1 ? 1 : occ);
  k->mat_block = MAT_BLOCK;
  k->mat_smem = materialize_smem_bytes(W, NP);
  int mocc = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mocc, materialize_kernel<W>, MAT_BLOCK,
                                                k->mat_smem);
  if (mocc < 1) mocc = 1;
  k->mat_grid = num_sms * mocc;
  k->red_block = RED_BLOCK;
  int rocc = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rocc, reduce_kernel<W>, RED_BLOCK, 0);
  if (rocc < 1) rocc = 1;
  k->red_grid = num_sms * rocc;
}

bool level_kernel_info(uint32_t W, uint32_t NP, int num_sms, LevelKernelInfo* out) {
  switch (W) {
    case 1: fill_info<1>(num_sms, NP, out); return true;
    case 2: fill_info<2>(num_sms, NP, out); return true;
    case 4: fill_info<4>(num_sms, NP, out); return true;
    case 8: fill_info<8>(num_sms, NP, out); return true;
    case 16: fill_info<16>(num_sms, NP, out); return true;
    case 32: fill_info<32>(num_sms, NP, out); return true;
    case 64: fill_info<64>(num_sms, NP, out); return true;
    default: return false;
  }
}

template <int W>
static void launch_init_t(const LevelParams& p, cudaStream_t s) {
  init_kernel<W><<<1, 256, 0, s>>>(p);
}
void launch_init(const LevelParams& p, cudaStream_t s) {
  switch (p.W) {
    case 1: launch_init_t<1>(p, s); break;
    case 2: launch_init_t<2>(p, s); break;
    case 4: launch_init_t<4>(p, s); break;
    case 8: launch_init_t<8>(p, s); break;
    case 16: launch_init_t<16>(p, s); break;
    case 32: launch_init_t<32>(p, s); break;
    case 64: launch_init_t<64>(p, s); break;
  }
}

template <int W, bool COUNT>
static void launch_level_t(const LevelParams& p, const LevelKernelInfo& k, uint32_t dir,
                           cudaStream_t s) {
  const cudaGraphConditionalHandle none = 0;
  if (dir != DIR_PUSH)
    level_kernel<W, DIR_PULL, COUNT><<<k.level_grids[DIR_PULL], k.level_block, 0, s>>>(p, none);
  if (dir != DIR_PULL)
    level_kernel<W, DIR_PUSH, COUNT><<<k.level_grids[DIR_PUSH], k.level_block, 0, s>>>(p, none);
}
template <int W>
static void launch_level_w(const LevelParams& p, const LevelKernelInfo& k, uint32_t dir,
                           bool count, cudaStream_t s) {
  if (count)
    launch_level_t<W, true>(p, k, dir, s);
  else
    launch_level_t<W, false>(p, k, dir, s);
}
void launch_level(const LevelParams& p, const LevelKernelInfo& k, uint32_t dir, bool count,
                  cudaStream_t s) {
  switch (p.W) {
    case 1: launch_level_w<1>(p, k, dir, count, s); break;
    case 2: launch_level_w<2>(p, k, dir, count, s); break;
    case 4: launch_level_w<4>(p, k, dir, count, s); break;
    case 8: launch_level_w<8>(p, k, dir, count, s); break;
    case 16: launch_level_w<16>(p, k, dir, count, s); break;
    case 32: launch_level_w<32>(p, k, dir, count, s); break;
    case 64: launch_level_w<64>(p, k, dir, count, s); break;
  }
}

template <int W>
static void launch_mat_t(const LevelParams& p, const LevelKernelInfo& k, bool reduce,
                         cudaStream_t s, uint32_t phase) {
  if (reduce)
    reduce_kernel<W><<<k.red_grid, k.red_block, 0, s>>>(p);
  else
    materialize_kernel<W><<<k.mat_grid, k.mat_block, k.mat_smem, s>>>(p, phase);
}
void launch_materialize(const LevelParams& p, const LevelKernelInfo& k, bool reduce,
                        cudaStream_t s, uint32_t phase) {
  switch (p.W) {
    case 1: launch_mat_t<1>(p, k, reduce, s, phase); break;
    case 2: launch_mat_t<2>(p, k, reduce, s, phase); break;
    case 4: launch_mat_t<4>(p, k, reduce, s, phase); break;
    case 8: launch_mat_t<8>(p, k, reduce, s, phase); break;
    case 16: launch_mat_t<16>(p, k, reduce, s, phase); break;
    case 32: launch_mat_t<32>(p, k, reduce, s, phase); break;
    case 64: launch_mat_t<64>(p, k, reduce, s, phase); break;
  }
}

template <int W>
static void launch_cleanup_t(const LevelParams& p, cudaStream_t s) {
  cleanup_kernel<W><<<256, 256, 0, s>>>(p);
}
void launch_cleanup(const LevelParams& p, cudaStream_t s) {
  switch (p.W) {
    case 1: launch_cleanup_t<1>(p, s); break;
    case 2: launch_cleanup_t<2>(p, s); break;
    case 4: launch_cleanup_t<4>(p, s); break;
    case 8: launch_cleanup_t<8>(p, s); break;
    case 16: launch_cleanup_t<16>(p, s); break;
    case 32: launch_cleanup_t<32>(p, s); break;
    case 64: launch_cleanup_t<64>(p, s); break;
  }
}

void launch_traversed_edges(uint32_t V, const uint32_t* off, const uint32_t* dist,
                            uint32_t num_sources, unsigned long long* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  traversed_edges_kernel<<<1024, 256, 0, s>>>(V, off, dist, num_sources, out);
}

}  // namespace msbfs
