// Served form: a resident graph, a request queue and a scheduler thread that
// packs queued requests into the source lanes of shared traversals running
// on several slots (engines/streams) at once. See include/msbfs.h ("served
// form") for the contract. No reference counterpart: the reference answers
// one blocking query per call (crates/gpu_bfs/src/engine.rs:219-298).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/msbfs.h"

// engine.cu: lets a second engine of the device run on a resident graph.
int msbfs_graph_attach(msbfs_graph* g, msbfs_engine* e);

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  std::vector<uint32_t> src;
  int mode = MSBFS_SERVE_STATS;
  void* out = nullptr;
  bool out_pinned = false;   // device-visible page-locked host memory
  size_t next = 0;           // first source not yet given to a launch
  size_t in_flight = 0;      // launches of this request still running
  uint32_t launches = 0;
  bool launched = false;
  bool done = false;
  int status = MSBFS_OK;
  Clock::time_point submit, first_launch, complete;
};

struct Part {
  Request* r;
  size_t src_off;   // first source of the request in this launch
  size_t n;
  size_t lane_off;  // its first lane in the launch
};

struct Slot {
  msbfs_engine* eng = nullptr;
  msbfs_graph* g = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  size_t rows_off = 0;    // the running launch's rows in the server's pool
  size_t rows_bytes = 0;  // (0: none reserved)
  msbfs_source_stats* d_stats = nullptr;
  void* h_stage = nullptr;  // page-locked bounce buffer for pageable outputs
  size_t h_stage_bytes = 0;
  std::vector<Part> parts;
  int mode = MSBFS_SERVE_STATS;
  bool express = false;  // takes small requests only, narrow launches
  bool busy = false;
  int launch_rc = MSBFS_OK;
};

size_t elem_bytes(int mode, size_t V) {
  return mode == MSBFS_SERVE_ROWS ? V * sizeof(uint32_t) : sizeof(msbfs_source_stats);
}

// First-fit allocator over the server's device pool for distance rows, with
// coalescing of freed ranges. Admission asks it for the largest free range
// before packing a launch, so a launch never needs more bytes than exist.
class RowPool {
 public:
  void reset(size_t bytes) {
    free_.clear();
    if (bytes) free_[0] = bytes;
  }
  size_t largest() const {
    size_t m = 0;
    for (const auto& kv : free_) m = std::max(m, kv.second);
    return m;
  }
  bool alloc(size_t bytes, size_t* off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, at = it->first + bytes;
      free_.erase(it);
      if (rest) free_[at] = rest;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<size_t, size_t> free_;  // offset -> bytes
};

}  // namespace

struct msbfs_server {
  int device = 0;
  size_t V = 0;
  msbfs_server_config cfg{};
  msbfs_graph* graph = nullptr;  // resident once, owned by slot 0's engine
  char* d_pool = nullptr;        // hbm_budget_bytes of distance-row staging
  RowPool pool;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_id = 1;
  bool stop = false;
  uint64_t traversals = 0, kernel_launches = 0;
  std::thread sched;
};

namespace {

void finish_part(msbfs_server* s, const Part& p, int rc) {
  Request* r = p.r;
  if (rc && !r->status) r->status = rc;
  if (--r->in_flight == 0 && r->next == r->src.size()) {
    r->done = true;
    r->complete = Clock::now();
    s->cv_done.notify_all();
  }
}

// Issues one launch on slot `sl` (called without the lock; the slot is busy
// so only the scheduler touches it).
int launch_slot(msbfs_server* s, Slot& sl, const std::vector<uint32_t>& lanes) {
  const size_t V = s->V, n = lanes.size();
  const size_t eb = elem_bytes(sl.mode, V);
  int rc;
  uint32_t* d_rows = reinterpret_cast<uint32_t*>(s->d_pool + sl.rows_off);
  if (sl.mode == MSBFS_SERVE_ROWS)
    rc = msbfs_run_ms_bfs_device(sl.eng, s->cfg.method, sl.g, lanes.data(), n, d_rows);
  else
    rc = msbfs_run_ms_bfs_stats_device(sl.eng, s->cfg.method, sl.g, lanes.data(), n,
                                       sl.d_stats);
  if (rc) return rc;
  bool need_stage = false;
  for (const Part& p : sl.parts) need_stage |= !p.r->out_pinned;
  if (need_stage && sl.h_stage_bytes < n * eb) {
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    sl.h_stage = nullptr;
    sl.h_stage_bytes = 0;
    if (cudaMallocHost(&sl.h_stage, n * eb) != cudaSuccess) {
      cudaGetLastError();
      return MSBFS_ERR_OOM;
    }
    sl.h_stage_bytes = n * eb;
  }
  const char* dsrc = sl.mode == MSBFS_SERVE_ROWS ? reinterpret_cast<const char*>(d_rows)
                                                 : reinterpret_cast<const char*>(sl.d_stats);
  for (const Part& p : sl.parts) {
    char* dst = p.r->out_pinned ? static_cast<char*>(p.r->out) + p.src_off * eb
                                : static_cast<char*>(sl.h_stage) + p.lane_off * eb;
    if (cudaMemcpyAsync(dst, dsrc + p.lane_off * eb, p.n * eb, cudaMemcpyDeviceToHost,
                        sl.stream) != cudaSuccess) {
      cudaGetLastError();
      return MSBFS_ERR_CUDA;
    }
  }
  if (cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return MSBFS_ERR_CUDA;
  }
  return MSBFS_OK;
}

void scheduler(msbfs_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progress = false, any_busy = false;
    // Completions: results are in host memory once the slot's event fired.
    for (Slot& sl : s->slots) {
      if (!sl.busy) continue;
      int rc = sl.launch_rc;
      if (!rc) {
        const cudaError_t q = cudaEventQuery(sl.ev);
        if (q == cudaErrorNotReady) {
          any_busy = true;
          continue;
        }
        if (q != cudaSuccess) {
          cudaGetLastError();
          rc = MSBFS_ERR_CUDA;
        }
      }
      if (!rc) {
        // Already complete: collects the traversal's status and level count.
        msbfs_stats st{};
        rc = msbfs_engine_synchronize(sl.eng, &st);
        s->traversals++;
        s->kernel_launches +=
            st.path == MSBFS_PATH_CTA ? 1 : (uint64_t)(st.levels + 3) * st.passes;
      }
      const size_t eb = elem_bytes(sl.mode, s->V);
      for (const Part& p : sl.parts) {
        if (!rc && !p.r->out_pinned)
          std::memcpy(static_cast<char*>(p.r->out) + p.src_off * eb,
                      static_cast<char*>(sl.h_stage) + p.lane_off * eb, p.n * eb);
        finish_part(s, p, rc);
      }
      sl.parts.clear();
      if (sl.rows_bytes) s->pool.release(sl.rows_off, sl.rows_bytes);
      sl.rows_bytes = 0;
      sl.busy = false;
      progress = true;
    }
    // Admissions: the next free slot takes queued requests of one output
    // mode, in arrival order, until its lanes are used up -- and, for rows,
    // until the lanes' rows (V u32 each) fill the largest free range of the
    // server's row pool, which the launch then reserves until it completes;
    // larger requests continue in later launches. An express slot takes
    // small requests only; a general slot takes large requests first when
    // express slots exist, small ones only when no large request waits.
    const size_t small = s->cfg.small_sources;
    for (Slot& sl : s->slots) {
      if (sl.busy || s->queue.empty()) continue;
      const bool have_express = s->cfg.express_slots > 0;
      bool want_small = sl.express;
      const Request* head = nullptr;
      for (const Request* r : s->queue) {
        const bool is_small = r->src.size() <= small;
        if (sl.express ? is_small : (!have_express || !is_small)) {
          head = r;
          break;
        }
      }
      if (!head && !sl.express) {  // no large request waits: take small ones
        head = s->queue.front();
        want_small = true;
      }
      if (!head) continue;
      sl.mode = head->mode;
      size_t cap = s->cfg.max_sources_per_launch;
      if (sl.express) cap = std::min(cap, 2 * small);
      const size_t row_bytes = s->V * sizeof(uint32_t);
      if (sl.mode == MSBFS_SERVE_ROWS) {
        cap = std::min(cap, s->pool.largest() / row_bytes);
        if (cap == 0) continue;  // rows of a single lane do not fit until a launch completes
      }
      std::vector<uint32_t> lanes;
      const auto now = Clock::now();
      for (size_t i = 0; i < s->queue.size() && lanes.size() < cap;) {
        Request* r = s->queue[i];
        const bool is_small = r->src.size() <= small;
        const bool eligible = sl.express ? is_small
                              : (!have_express || want_small) ? true
                                                              : !is_small;
        if (r->mode != sl.mode || !eligible) {
          ++i;
          continue;
        }
        const size_t left = r->src.size() - r->next;
        if (sl.express && !lanes.empty() && left > cap - lanes.size()) {
          ++i;  // a small request is not split while a later launch can hold it whole
          continue;
        }
        const size_t take = std::min(left, cap - lanes.size());
        sl.parts.push_back(Part{r, r->next, take, lanes.size()});
        lanes.insert(lanes.end(), r->src.begin() + r->next, r->src.begin() + r->next + take);
        r->next += take;
        r->in_flight++;
        r->launches++;
        if (!r->launched) {
          r->launched = true;
          r->first_launch = now;
        }
        if (r->next == r->src.size())
          s->queue.erase(s->queue.begin() + i);
        else
          ++i;
      }
      // The pool's largest range held `cap` lanes' rows a moment ago and
      // only this thread allocates, so the reservation succeeds.
      bool reserved = true;
      sl.rows_bytes = 0;
      if (sl.mode == MSBFS_SERVE_ROWS) {
        reserved = s->pool.alloc(lanes.size() * row_bytes, &sl.rows_off);
        if (reserved) sl.rows_bytes = lanes.size() * row_bytes;
      }
      sl.busy = true;
      any_busy = true;
      progress = true;
      lk.unlock();
      sl.launch_rc = reserved ? launch_slot(s, sl, lanes) : MSBFS_ERR_OOM;
      lk.lock();
    }
    if (s->stop && s->queue.empty() && !any_busy) break;
    if (!progress)
      s->cv_work.wait_for(lk, any_busy ? std::chrono::microseconds(20)
                                       : std::chrono::microseconds(2000));
  }
}

void destroy_slots(msbfs_server* s) {
  for (Slot& sl : s->slots)
    if (sl.stream) cudaStreamSynchronize(sl.stream);
  // The shared graph goes first: it drops every attached engine's workspaces.
  if (s->graph) msbfs_graph_destroy(s->graph);
  s->graph = nullptr;
  if (s->d_pool) cudaFree(s->d_pool);
  s->d_pool = nullptr;
  for (Slot& sl : s->slots) {
    if (sl.eng) msbfs_engine_destroy(sl.eng);
    if (sl.d_stats) cudaFree(sl.d_stats);
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  s->slots.clear();
}

}  // namespace

extern "C" {

int msbfs_server_create(int device, size_t V, size_t E, const uint32_t* ro, const uint32_t* ci,
                        const msbfs_server_config* config, msbfs_server** out) {
  if (!out) return MSBFS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (V == 0) return MSBFS_ERR_EMPTY_GRAPH;
  auto s = std::make_unique<msbfs_server>();
  s->device = device;
  s->V = V;
  if (config) s->cfg = *config;
  if (!config) s->cfg.method = MSBFS_METHOD_AUTO;
  if (s->cfg.slots == 0) s->cfg.slots = 2;
  if (s->cfg.max_sources_per_launch == 0) s->cfg.max_sources_per_launch = 512;
  if (s->cfg.hbm_budget_bytes == 0) s->cfg.hbm_budget_bytes = 8ull << 30;
  if (s->cfg.small_sources == 0) s->cfg.small_sources = 64;
  if (s->cfg.general_sm_percent == 0) s->cfg.general_sm_percent = 100;
  if (s->cfg.method < 0 || s->cfg.method > MSBFS_METHOD_AUTO ||
      s->cfg.express_slots >= s->cfg.slots || s->cfg.general_sm_percent > 100 ||
      s->cfg.reserved != 0)
    return MSBFS_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return MSBFS_ERR_NO_DEVICE;
  }
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  // The row pool holds at least one lane's rows.
  const size_t pool_bytes = std::max<size_t>(s->cfg.hbm_budget_bytes / (V * 4), 1) * V * 4;
  if (cudaMalloc((void**)&s->d_pool, pool_bytes) != cudaSuccess) {
    cudaGetLastError();
    return MSBFS_ERR_OOM;
  }
  s->pool.reset(pool_bytes);
  s->slots.resize(s->cfg.slots);
  int rc = MSBFS_OK;
  for (size_t k = 0; k < s->slots.size(); ++k) {
    Slot& sl = s->slots[k];
    sl.express = k < s->cfg.express_slots;
    if ((rc = msbfs_engine_create(device, s->cfg.method, &sl.eng))) break;
    if (cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking,
                                     sl.express ? prio_high : prio_low) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
      rc = MSBFS_ERR_CUDA;
      break;
    }
    if ((rc = msbfs_engine_set_stream(sl.eng, sl.stream))) break;
    if (!sl.express && s->cfg.general_sm_percent < 100 &&
        (rc = msbfs_engine_set_sm_share(sl.eng, s->cfg.general_sm_percent)))
      break;
    // A general slot's launch is one pass as wide as its lanes (up to 64
    // words, 2,048 lanes): one wide pass costs far less per source than
    // several 512-lane passes (R-MAT scale 24, per-source statistics, 2,048
    // sources: 94 ms in one pass, 174 ms in four).
    if (!sl.express && s->cfg.max_sources_per_launch > 512) {
      uint32_t words = 1;
      while (words * 32 < s->cfg.max_sources_per_launch && words < 64) words <<= 1;
      if ((rc = msbfs_engine_set_tuning(sl.eng, words, 0, 0))) break;
    }
    // One resident copy of the graph, shared by every slot's engine.
    if (k == 0 && (rc = msbfs_graph_create(sl.eng, V, E, ro, ci, &s->graph))) break;
    if ((rc = msbfs_graph_attach(s->graph, sl.eng))) break;
    sl.g = s->graph;
    if (cudaMalloc((void**)&sl.d_stats,
                   s->cfg.max_sources_per_launch * sizeof(msbfs_source_stats)) != cudaSuccess) {
      cudaGetLastError();
      rc = MSBFS_ERR_OOM;
      break;
    }
  }
  if (rc) {
    destroy_slots(s.get());
    return rc;
  }
  msbfs_server* raw = s.get();
  s->sched = std::thread(scheduler, raw);
  *out = s.release();
  return MSBFS_OK;
}

int msbfs_server_submit(msbfs_server* s, const uint32_t* sources, size_t S, int mode, void* out,
                        uint64_t* ticket) {
  if (!s || !ticket || (S && (!sources || !out))) return MSBFS_ERR_INVALID_ARGUMENT;
  if (mode != MSBFS_SERVE_ROWS && mode != MSBFS_SERVE_STATS) return MSBFS_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < S; ++i)
    if ((size_t)sources[i] >= s->V) return MSBFS_ERR_SOURCE_OOB;
  auto r = std::make_unique<Request>();
  r->src.assign(sources, sources + S);
  r->mode = mode;
  r->out = out;
  cudaPointerAttributes attr{};
  if (out && cudaPointerGetAttributes(&attr, out) == cudaSuccess &&
      attr.type == cudaMemoryTypeHost)
    r->out_pinned = true;
  else
    cudaGetLastError();
  r->submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return MSBFS_ERR_INVALID_ARGUMENT;
  r->id = s->next_id++;
  *ticket = r->id;
  if (S == 0) {
    r->done = true;
    r->complete = r->first_launch = r->submit;
  } else {
    s->queue.push_back(r.get());
  }
  s->reqs[r->id] = std::move(r);
  s->cv_work.notify_one();
  return MSBFS_OK;
}

int msbfs_server_wait(msbfs_server* s, uint64_t ticket, double timeout_ms,
                      msbfs_request_info* info) {
  if (!s) return MSBFS_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return MSBFS_ERR_INVALID_ARGUMENT;
  Request* r = it->second.get();
  auto pred = [r] { return r->done; };
  if (timeout_ms < 0)
    s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred))
    return MSBFS_ERR_TIMEOUT;
  const int st = r->status;
  if (info) {
    using ms = std::chrono::duration<double, std::milli>;
    info->latency_ms = ms(r->complete - r->submit).count();
    info->queue_ms = ms(r->first_launch - r->submit).count();
    info->launches = r->launches;
    info->status = st;
  }
  s->reqs.erase(it);
  return st;
}

int msbfs_server_counters(msbfs_server* s, uint64_t* traversals, uint64_t* kernel_launches) {
  if (!s) return MSBFS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  if (traversals) *traversals = s->traversals;
  if (kernel_launches) *kernel_launches = s->kernel_launches;
  return MSBFS_OK;
}

void msbfs_server_destroy(msbfs_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->sched.joinable()) s->sched.join();
  cudaSetDevice(s->device);
  destroy_slots(s);
  delete s;
}

}  // extern "C"
