/*
 * CPU oracle for the multi-source BFS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's CPU BFS paths (crates/cpu_bfs) and
 * graph helpers (crates/core/src/graph.rs). Used by the tests, the smoke check
 * and the CPU-baseline leg of the benchmark as the checker; the CUDA engine
 * never links it. See oracle.h for how the restatement is pinned.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define DIST_MAX 0xFFFFFFFFu

/* fifo.rs:10-46: queue-cursor BFS, claim on dist == MAX, CSR order. */
void oracle_bfs_single_source_into(size_t V, const uint32_t *ro,
                                   const uint32_t *ci, uint32_t source,
                                   uint32_t *dist, uint32_t *queue) {
  if (V == 0) return;
  dist[source] = 0;
  size_t head = 0, tail = 0;
  queue[tail++] = source;
  while (head < tail) {
    uint32_t u = queue[head++];
    uint32_t nd = dist[u] + 1;
    for (uint32_t e = ro[u]; e < ro[u + 1]; ++e) {
      uint32_t v = ci[e];
      if (dist[v] == DIST_MAX) {
        dist[v] = nd;
        queue[tail++] = v;
      }
    }
  }
}

/* Up-front validation shared by fifo.rs:80-90, rayon_ms.rs:20-29 and
 * bit_parallel.rs:110-120: the first source >= V is reported with its index. */
static int validate_sources(size_t V, const uint32_t *sources, size_t S,
                            size_t *bad_index) {
  for (size_t i = 0; i < S; ++i) {
    if ((size_t)sources[i] >= V) {
      if (bad_index) *bad_index = i;
      return ORACLE_ERR_SOURCE_OOB;
    }
  }
  return ORACLE_OK;
}

/* fifo.rs:70-102. */
int oracle_ms_bfs_fifo(size_t V, const uint32_t *ro, const uint32_t *ci,
                       const uint32_t *sources, size_t S, uint32_t *out,
                       size_t *bad_index) {
  if (S == 0 || V == 0) return ORACLE_OK;
  int rc = validate_sources(V, sources, S, bad_index);
  if (rc) return rc;
  memset(out, 0xFF, S * V * sizeof(uint32_t));
  uint32_t *queue = (uint32_t *)malloc(V * sizeof(uint32_t));
  if (!queue) return ORACLE_ERR_INVALID;
  for (size_t s = 0; s < S; ++s)
    oracle_bfs_single_source_into(V, ro, ci, sources[s], out + s * V, queue);
  free(queue);
  return ORACLE_OK;
}

/* rayon_ms.rs:11-54: one FIFO BFS per source, rows are disjoint so the
 * threads share nothing but the read-only graph. Sources are handed out by an
 * atomic cursor (the reference uses Rayon's work stealing; the output does
 * not depend on the schedule). */
typedef struct {
  size_t V, S;
  const uint32_t *ro, *ci, *sources;
  uint32_t *out;
  size_t next;
} threaded_job;

static void *threaded_worker(void *arg) {
  threaded_job *job = (threaded_job *)arg;
  uint32_t *queue = (uint32_t *)malloc(job->V * sizeof(uint32_t));
  if (!queue) return NULL;
  for (;;) {
    size_t s = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
    if (s >= job->S) break;
    uint32_t *row = job->out + s * job->V;
    memset(row, 0xFF, job->V * sizeof(uint32_t));
    oracle_bfs_single_source_into(job->V, job->ro, job->ci, job->sources[s],
                                  row, queue);
  }
  free(queue);
  return NULL;
}

int oracle_ms_bfs_threaded(size_t V, const uint32_t *ro, const uint32_t *ci,
                           const uint32_t *sources, size_t S, uint32_t *out,
                           int threads, size_t *bad_index) {
  if (S == 0 || V == 0) return ORACLE_OK;
  int rc = validate_sources(V, sources, S, bad_index);
  if (rc) return rc;
  if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (threads < 1) threads = 1;
  if ((size_t)threads > S) threads = (int)S;
  threaded_job job = {V, S, ro, ci, sources, out, 0};
  pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  if (!tids) return ORACLE_ERR_INVALID;
  for (int t = 0; t < threads; ++t)
    pthread_create(&tids[t], NULL, threaded_worker, &job);
  for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
  free(tids);
  return ORACLE_OK;
}

/* bit_parallel.rs:11-97: one batch of <= 64 sources. `frontier`, `seen` and
 * `next_frontier` are u64 per vertex; active lists hold touched vertices. */
static void bit_parallel_batch_64(size_t V, const uint32_t *ro,
                                  const uint32_t *ci, const uint32_t *batch,
                                  size_t batch_size, size_t batch_start,
                                  uint32_t *dist, uint64_t *seen,
                                  uint64_t *frontier, uint64_t *next_frontier,
                                  uint32_t *active, uint32_t *next_active) {
  memset(seen, 0, V * sizeof(uint64_t));
  memset(frontier, 0, V * sizeof(uint64_t));
  memset(next_frontier, 0, V * sizeof(uint64_t));
  size_t n_active = 0, n_next = 0;
  for (size_t k = 0; k < batch_size; ++k) {
    uint32_t s = batch[k];
    uint64_t mask = 1ull << k;
    dist[(batch_start + k) * V + s] = 0;
    if (frontier[s] == 0) active[n_active++] = s;
    frontier[s] |= mask;
    seen[s] |= mask;
  }
  uint32_t cur = 0;
  while (n_active) {
    uint32_t nd = cur + 1;
    for (size_t i = 0; i < n_active; ++i) {
      uint32_t u = active[i];
      uint64_t f = frontier[u];
      frontier[u] = 0;
      for (uint32_t e = ro[u]; e < ro[u + 1]; ++e) {
        uint32_t v = ci[e];
        if (next_frontier[v] == 0) next_active[n_next++] = v;
        next_frontier[v] |= f;
      }
    }
    n_active = 0;
    for (size_t i = 0; i < n_next; ++i) {
      uint32_t v = next_active[i];
      uint64_t nf = next_frontier[v];
      next_frontier[v] = 0;
      uint64_t nv = nf & ~seen[v];
      if (nv) {
        seen[v] |= nv;
        frontier[v] = nv;
        active[n_active++] = v;
        while (nv) {
          int b = __builtin_ctzll(nv);
          dist[(batch_start + (size_t)b) * V + v] = nd;
          nv &= nv - 1;
        }
      }
    }
    n_next = 0;
    cur++;
  }
}

/* bit_parallel.rs:101-130. The reference's next_active list can hold a vertex
 * once per level (guarded by next_frontier[v] == 0), so V entries suffice. */
int oracle_ms_bfs_bit_parallel(size_t V, const uint32_t *ro, const uint32_t *ci,
                               const uint32_t *sources, size_t S, uint32_t *out,
                               size_t *bad_index) {
  if (S == 0 || V == 0) return ORACLE_OK;
  int rc = validate_sources(V, sources, S, bad_index);
  if (rc) return rc;
  memset(out, 0xFF, S * V * sizeof(uint32_t));
  uint64_t *seen = (uint64_t *)malloc(V * sizeof(uint64_t));
  uint64_t *fr = (uint64_t *)malloc(V * sizeof(uint64_t));
  uint64_t *nf = (uint64_t *)malloc(V * sizeof(uint64_t));
  uint32_t *act = (uint32_t *)malloc(V * sizeof(uint32_t));
  uint32_t *nact = (uint32_t *)malloc(V * sizeof(uint32_t));
  if (!seen || !fr || !nf || !act || !nact) {
    free(seen); free(fr); free(nf); free(act); free(nact);
    return ORACLE_ERR_INVALID;
  }
  for (size_t b = 0; b < S; b += 64) {
    size_t n = S - b < 64 ? S - b : 64;
    bit_parallel_batch_64(V, ro, ci, sources + b, n, b, out, seen, fr, nf, act,
                          nact);
  }
  free(seen); free(fr); free(nf); free(act); free(nact);
  return ORACLE_OK;
}

/* graph.rs:571-646 (sequential form of the Rayon loop). */
void oracle_reachability_from_distances(size_t V, size_t S, const uint32_t *dist,
                                        uint32_t *words) {
  if (S == 0 || V == 0) return;
  size_t wpv = (S + 31) / 32;
  for (size_t v = 0; v < V; ++v)
    for (size_t w = 0; w < wpv; ++w) {
      uint32_t word = 0;
      size_t s0 = w * 32, n = S - s0 < 32 ? S - s0 : 32;
      for (size_t b = 0; b < n; ++b)
        if (dist[(s0 + b) * V + v] != DIST_MAX) word |= 1u << b;
      words[v * wpv + w] = word;
    }
}

/* crates/cli/src/bench.rs:478-491. */
uint64_t oracle_traversed_edges(size_t V, const uint32_t *ro, size_t S,
                                const uint32_t *dist) {
  uint64_t total = 0;
  for (size_t s = 0; s < S; ++s)
    for (size_t u = 0; u < V; ++u)
      if (dist[s * V + u] != DIST_MAX) total += ro[u + 1] - ro[u];
  return total;
}

static int cmp_edge(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* graph.rs:51-88: filter, sort_unstable, dedup, count, prefix-sum. */
void oracle_csr_from_edge_list(size_t V, size_t n_edges, const uint32_t *eu,
                               const uint32_t *ev, uint32_t *ro, uint32_t *ci,
                               size_t *out_E) {
  uint64_t *keys = (uint64_t *)malloc((n_edges ? n_edges : 1) * sizeof(uint64_t));
  size_t n = 0;
  for (size_t i = 0; i < n_edges; ++i)
    if (eu[i] != ev[i] && (size_t)eu[i] < V && (size_t)ev[i] < V)
      keys[n++] = ((uint64_t)eu[i] << 32) | ev[i];
  qsort(keys, n, sizeof(uint64_t), cmp_edge);
  size_t m = 0;
  for (size_t i = 0; i < n; ++i)
    if (m == 0 || keys[i] != keys[m - 1]) keys[m++] = keys[i];
  memset(ro, 0, (V + 1) * sizeof(uint32_t));
  for (size_t i = 0; i < m; ++i) ro[(keys[i] >> 32) + 1]++;
  for (size_t i = 0; i < V; ++i) ro[i + 1] += ro[i];
  for (size_t i = 0; i < m; ++i) ci[i] = (uint32_t)keys[i];
  *out_E = m;
  free(keys);
}

/* graph.rs:90-127: in-degree count, prefix sum, scatter in row order. */
void oracle_to_csc(size_t V, size_t E, const uint32_t *ro, const uint32_t *ci,
                   uint32_t *co, uint32_t *ri) {
  memset(co, 0, (V + 1) * sizeof(uint32_t));
  for (size_t e = 0; e < E; ++e) co[ci[e] + 1]++;
  for (size_t i = 0; i < V; ++i) co[i + 1] += co[i];
  uint32_t *pos = (uint32_t *)malloc((V ? V : 1) * sizeof(uint32_t));
  memcpy(pos, co, V * sizeof(uint32_t));
  for (size_t u = 0; u < V; ++u)
    for (uint32_t e = ro[u]; e < ro[u + 1]; ++e) ri[pos[ci[e]]++] = (uint32_t)u;
  free(pos);
}

/* graph.rs:129-133. */
int oracle_is_symmetric(size_t V, size_t E, const uint32_t *ro,
                        const uint32_t *ci) {
  uint32_t *co = (uint32_t *)malloc((V + 1) * sizeof(uint32_t));
  uint32_t *ri = (uint32_t *)malloc((E ? E : 1) * sizeof(uint32_t));
  oracle_to_csc(V, E, ro, ci, co, ri);
  int sym = memcmp(co, ro, (V + 1) * sizeof(uint32_t)) == 0 &&
            (E == 0 || memcmp(ri, ci, E * sizeof(uint32_t)) == 0);
  free(co);
  free(ri);
  return sym;
}
