// Serving loop: continuous batching of CLUE 2D events (no reference
// counterpart; the reference runs a fixed set of events per EDM stream,
// src/serial/bin/StreamSchedule.cc:61-93).
//
// Requests are queued by clue_server_submit (inputs copied on submit).  A
// scheduler thread owns `max_inflight` slots; each slot is a CLUE handle with
// its own CUDA stream, resident device buffers and pinned staging.  At start
// every slot sizes its buffers for batches of up to 8M points within half of
// an equal share of the budget, so that ordinary loads never allocate.
// Whenever a slot is free and requests are waiting, the scheduler admits as
// many queued events as fit those buffers (points and event count), stages
// them, and launches the batched pipeline asynchronously; batches of different
// slots overlap on the device (one batch's copies with another's kernels).
// An event larger than a start-up batch goes alone and may take the rest of
// the shared budget: it is admitted when the slots' device memory together
// stays within the budget -- idle slots first give back what they grew beyond
// their start-up buffers -- and otherwise waits, at the head of the queue,
// until in-flight batches finish.  Only an event that cannot fit even when
// every other slot holds just its start-up buffers is refused (CLUE_ENOMEM).
// Completed batches are found with cudaEventQuery (every 20 us while batches
// are in flight), their outputs are copied to each caller's buffers, and the
// request latency (submit -> outputs written) is recorded.  Host copies run
// on a resident pool.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/clue.h"
#include "clue_internal.h"
#include "clue_runtime.h"
#include "copy_pool.h"

namespace clue {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int32_t n = 0;
  std::vector<float> x, y, w;
  std::vector<int32_t> layer;
  clue_outputs out{};
  Clock::time_point t_submit;
  double latency_ms = 0.0;
  int status = CLUE_EBUSY;
};

struct Slot {
  clue_handle* h = nullptr;
  PinnedBuf in, out;
  std::vector<int64_t> off;
  std::vector<Request*> reqs;
  bool busy = false;      // requests taken (staging, on the device or delivering results)
  bool launched = false;  // the batch is queued on the device
  int64_t batch_points = 0;  // batches are cut at this size: the buffers sized at start
  size_t base_bytes = 0;     // device bytes of those start-up buffers
};

class Server {
 public:
  Server(const clue_params& p, const clue_server_config& c) : params_(p), cfg_(c) {}
  ~Server() { shutdown(); }

  int start() {
    if (cfg_.max_inflight < 1) cfg_.max_inflight = 1;
    if (cfg_.max_batch_events < 1) cfg_.max_batch_events = 1;
    if (!cfg_.device_budget_bytes) cfg_.device_budget_bytes = size_t(16) << 30;
    budget_ = cfg_.device_budget_bytes;
    // start-up buffers within half of an equal share: the other half of the
    // budget stays free for events larger than a start-up batch
    const size_t base_share = budget_ / (2 * (size_t)cfg_.max_inflight);
    slots_.resize(cfg_.max_inflight);
    for (auto& s : slots_) {
      int rc = clue_create(&params_, budget_, cfg_.device, nullptr, &s.h);
      if (rc) return rc;
      Handle* hh = reinterpret_cast<Handle*>(s.h);
      // largest batch (point count) whose buffers fit the start-up share
      int64_t lo = 0, hi = int64_t(1) << 31;
      const int grid = layer_grid_max(hh->tuning, cfg_.max_batch_events * kLayers);
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) / 2;
        const int64_t chunks = mid / kChunk + cfg_.max_batch_events;
        if (required_bytes_2d(cfg_.max_batch_events, mid, chunks, grid, true) <= base_share) lo = mid; else hi = mid;
      }
      if (lo < 1) return set_error(CLUE_ENOMEM, "budget too small for one in-flight batch");
      // resident buffers for batches up to 8M points, so that ordinary loads
      // never allocate (and never synchronise the device) on the serving path
      s.batch_points = std::min<int64_t>(lo, int64_t(8) << 20);
      cudaSetDevice(cfg_.device);
      rc = reserve_2d(hh, cfg_.max_batch_events, s.batch_points, true);
      if (!rc) rc = s.in.reserve(16 * (size_t)s.batch_points);
      if (!rc) rc = s.out.reserve(20 * (size_t)s.batch_points);
      if (rc) return rc;
      s.base_bytes = hh->arena.total();
    }
    // the largest single event ever admitted: it fits the budget while every
    // other slot holds only its start-up buffers
    const size_t others = (slots_.size() - 1) * slots_[0].base_bytes;
    const size_t room = budget_ > others ? budget_ - others : 0;
    const Handle* h0 = reinterpret_cast<const Handle*>(slots_[0].h);
    int64_t lo = 0, hi = int64_t(1) << 31;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) / 2;
      if (arena_bytes_after_2d(h0, 1, mid, mid / kChunk + 1, true) <= room) lo = mid; else hi = mid;
    }
    cap_points_ = lo;
    // helpers on all cores but two (the scheduler and a submitting client), at most 15
    pool_.start((int)std::min(15u, std::max(3u, std::thread::hardware_concurrency()) - 2));
    worker_ = std::thread([this] { loop(); });
    return CLUE_OK;
  }

  void shutdown() {
    {
      std::lock_guard<std::mutex> g(mu_);
      if (stop_) return;
      stop_ = true;
    }
    cv_.notify_all();
    if (worker_.joinable()) worker_.join();
    for (auto& s : slots_) {
      if (s.h) clue_destroy(s.h);
      s.h = nullptr;
    }
    for (auto& kv : reqs_) delete kv.second;
    reqs_.clear();
  }

  int submit(int32_t n, const float* x, const float* y, const int32_t* layer, const float* w,
             const clue_outputs* out, int64_t* id) {
    const int64_t off[2] = {0, n};
    if (n < 0) return set_error(CLUE_EINVAL, "bad argument");
    return submit_many(1, off, x, y, layer, w, out, id);
  }

  // Events enter the queue together, under one lock, so that the scheduler
  // can put them in one batch.
  int submit_many(int32_t E, const int64_t* off, const float* x, const float* y, const int32_t* layer,
                  const float* w, const clue_outputs* outs, int64_t* ids) {
    if (E < 0 || !outs || !ids || (E > 0 && (!off || off[0] != 0))) return set_error(CLUE_EINVAL, "bad argument");
    for (int32_t e = 0; e < E; ++e) {
      const int64_t n = off[e + 1] - off[e];
      if (n < 0 || n > INT32_MAX) return set_error(CLUE_EINVAL, "bad event_offsets");
      if (n > 0 && (!x || !y || !layer || !w)) return set_error(CLUE_EINVAL, "bad argument");
      if (n > cap_points_)
        return set_error(CLUE_ENOMEM,
                         "event of %lld points exceeds what the device budget admits (%lld points with the other "
                         "slots at their start-up buffers)",
                         (long long)n, (long long)cap_points_);
    }
    std::vector<Request*> rs(E);
    const auto now = Clock::now();
    std::vector<CopyTask> copies;
    copies.reserve(4 * (size_t)E);
    for (int32_t e = 0; e < E; ++e) {
      const int64_t s0 = off[e], n = off[e + 1] - s0;
      Request* r = new Request();
      r->n = (int32_t)n;
      if (n > 0) {
        r->x.resize(n);
        r->y.resize(n);
        r->w.resize(n);
        r->layer.resize(n);
        copies.push_back({r->x.data(), x + s0, 4 * (size_t)n});
        copies.push_back({r->y.data(), y + s0, 4 * (size_t)n});
        copies.push_back({r->w.data(), w + s0, 4 * (size_t)n});
        copies.push_back({r->layer.data(), layer + s0, 4 * (size_t)n});
      }
      r->out = outs[e];
      r->t_submit = now;
      rs[e] = r;
    }
    pool_.run(copies);
    {
      std::lock_guard<std::mutex> g(mu_);
      for (int32_t e = 0; e < E; ++e) {
        rs[e]->id = next_id_++;
        reqs_[rs[e]->id] = rs[e];
        queue_.push_back(rs[e]);
        ids[e] = rs[e]->id;
      }
    }
    cv_.notify_all();
    return CLUE_OK;
  }

  int poll(int64_t id, int32_t timeout_ms, double* lat) {
    std::unique_lock<std::mutex> g(mu_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return set_error(CLUE_EINVAL, "unknown request id %lld", (long long)id);
    Request* r = it->second;
    auto ready = [&] { return r->status != CLUE_EBUSY; };
    if (!ready()) {
      if (timeout_ms == 0) return CLUE_EBUSY;
      if (timeout_ms < 0) {
        done_cv_.wait(g, ready);
      } else if (!done_cv_.wait_for(g, std::chrono::milliseconds(timeout_ms), ready)) {
        return set_error(CLUE_ETIMEOUT, "request %lld not finished after %d ms", (long long)id, timeout_ms);
      }
    }
    const int st = r->status;
    if (lat) *lat = r->latency_ms;
    reqs_.erase(it);
    delete r;
    if (st != CLUE_OK) return set_error(st, "request %lld failed", (long long)id);
    return CLUE_OK;
  }

  int drain(int32_t timeout_ms) {
    std::unique_lock<std::mutex> g(mu_);
    auto idle = [&] {
      if (!queue_.empty()) return false;
      for (auto& s : slots_)
        if (s.busy) return false;
      return true;
    };
    if (timeout_ms < 0) {
      done_cv_.wait(g, idle);
    } else if (!done_cv_.wait_for(g, std::chrono::milliseconds(timeout_ms), idle)) {
      return set_error(CLUE_ETIMEOUT, "server not drained after %d ms", timeout_ms);
    }
    return CLUE_OK;
  }

  void stats(clue_server_stats* st) {
    std::lock_guard<std::mutex> g(mu_);
    st->completed = (int64_t)lat_.size();
    st->batches = batches_;
    std::vector<double> v = lat_;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
      if (v.empty()) return 0.0;
      size_t i = (size_t)std::min<double>(v.size() - 1, std::max(0.0, q * v.size() - 1e-9));
      return v[i];
    };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->mean_batch_events = batches_ ? double(batched_events_) / batches_ : 0.0;
    st->max_inflight_seen = max_inflight_seen_;
    st->slot_capacity_points = cap_points_;
    st->memory_waits = memory_waits_;
  }

  void reset_stats() {
    std::lock_guard<std::mutex> g(mu_);
    lat_.clear();
    batches_ = 0;
    batched_events_ = 0;
    max_inflight_seen_ = 0;
    memory_waits_ = 0;
  }

 private:
  size_t others_bytes(const Slot& s) const {
    size_t t = 0;
    for (const auto& o : slots_)
      if (&o != &s) t += reinterpret_cast<const Handle*>(o.h)->arena.total();
    return t;
  }

  // Completes every finished slot.  Called with mu_ held; the result copies
  // run with the lock released (only this thread touches slots), and the
  // statuses are published under the lock afterwards.
  bool reap(std::unique_lock<std::mutex>& g) {
    std::vector<Slot*> done;
    std::vector<int> sts;
    for (auto& s : slots_) {
      if (!s.busy || !s.launched) continue;
      Handle* h = reinterpret_cast<Handle*>(s.h);
      cudaError_t q = cudaEventQuery(h->done_event);
      if (q == cudaErrorNotReady) continue;
      int st = CLUE_OK;
      if (q != cudaSuccess) {
        st = cuda_error(q, "serving batch");
      } else {
        h->pending = false;
        st = h->check_device_flags();
      }
      done.push_back(&s);
      sts.push_back(st);
    }
    if (done.empty()) return false;
    g.unlock();
    std::vector<CopyTask> copies;
    for (size_t d = 0; d < done.size(); ++d) {
      Slot& s = *done[d];
      if (sts[d] != CLUE_OK) continue;
      const char* ob = static_cast<const char*>(s.out.p);
      const int64_t N = s.off.back();
      for (size_t k = 0; k < s.reqs.size(); ++k) {
        Request* r = s.reqs[k];
        const int64_t o = s.off[k];
        const size_t b = 4 * (size_t)r->n;
        if (r->n == 0) continue;
        copies.push_back({r->out.rho, ob + 4 * o, b});
        copies.push_back({r->out.delta, ob + 4 * (N + o), b});
        copies.push_back({r->out.nearestHigher, ob + 4 * (2 * N + o), b});
        copies.push_back({r->out.isSeed, ob + 4 * (3 * N + o), b});
        copies.push_back({r->out.clusterIndex, ob + 4 * (4 * N + o), b});
      }
    }
    pool_.run(copies);
    const auto now = Clock::now();
    g.lock();
    for (size_t d = 0; d < done.size(); ++d) {
      Slot& s = *done[d];
      for (Request* r : s.reqs) {
        r->latency_ms = std::chrono::duration<double, std::milli>(now - r->t_submit).count();
        r->status = sts[d];
        if (sts[d] == CLUE_OK) lat_.push_back(r->latency_ms);
      }
      s.reqs.clear();
      s.busy = false;
      s.launched = false;
    }
    done_cv_.notify_all();
    return true;
  }

  // Admits queued requests into a free slot and launches it.  Called with mu_
  // held; the requests are taken (and the slot marked busy, so that drain()
  // keeps waiting) under the lock, the staging copies and the launch run
  // without it.  Returns false when the head of the queue waits for device
  // memory (nothing is taken then).
  bool admit(Slot& s, std::unique_lock<std::mutex>& g) {
    s.reqs.clear();
    s.off.assign(1, 0);
    int64_t pts = 0, nchunks = 0;
    while (!queue_.empty() && (int)s.reqs.size() < cfg_.max_batch_events) {
      Request* r = queue_.front();
      // batches stay within the buffers sized at start (a single larger event
      // still goes, alone)
      if (pts + r->n > s.batch_points && !s.reqs.empty()) break;
      queue_.pop_front();
      s.reqs.push_back(r);
      pts += r->n;
      nchunks += (r->n + kChunk - 1) / kChunk;
      s.off.push_back(pts);
    }
    const int32_t E = (int32_t)s.reqs.size();
    if (E == 0) return true;
    Handle* hs = reinterpret_cast<Handle*>(s.h);
    // device memory of all slots together stays within the budget
    const size_t need = arena_bytes_after_2d(hs, E, pts, nchunks, true);
    size_t others = others_bytes(s);
    if (need + others > budget_) {
      // idle slots give back what they grew beyond their start-up buffers
      g.unlock();
      for (auto& o : slots_) {
        Handle* ho = reinterpret_cast<Handle*>(o.h);
        if (&o == &s || o.busy || ho->arena.total() <= o.base_bytes) continue;
        ho->arena.release();
        ho->budget = budget_;
        reserve_2d(ho, cfg_.max_batch_events, o.batch_points, true);
        o.base_bytes = ho->arena.total();
      }
      g.lock();
      others = others_bytes(s);
      if (need + others > budget_) {
        // the batch waits, in queue order, until in-flight batches finish
        for (int32_t k = E - 1; k >= 0; --k) queue_.push_front(s.reqs[k]);
        if (queue_.front()->id != waiting_id_) {
          waiting_id_ = queue_.front()->id;
          ++memory_waits_;
        }
        s.reqs.clear();
        s.off.assign(1, 0);
        return false;
      }
    }
    hs->budget = budget_ - others;  // the room this slot may grow into
    s.busy = true;
    g.unlock();
    int rc = s.in.reserve(16 * (size_t)std::max<int64_t>(pts, 1));
    if (!rc) rc = s.out.reserve(20 * (size_t)std::max<int64_t>(pts, 1));
    if (!rc) {
      char* ib = static_cast<char*>(s.in.p);
      std::vector<CopyTask> copies;
      copies.reserve(4 * (size_t)E);
      for (int32_t k = 0; k < E; ++k) {
        Request* r = s.reqs[k];
        const int64_t o = s.off[k];
        const size_t b = 4 * (size_t)r->n;
        if (r->n == 0) continue;
        copies.push_back({ib + 4 * o, r->x.data(), b});
        copies.push_back({ib + 4 * (pts + o), r->y.data(), b});
        copies.push_back({ib + 4 * (2 * pts + o), r->layer.data(), b});
        copies.push_back({ib + 4 * (3 * pts + o), r->w.data(), b});
      }
      pool_.run(copies);
      for (Request* r : s.reqs) {  // inputs are staged: free them now
        std::vector<float>().swap(r->x);
        std::vector<float>().swap(r->y);
        std::vector<float>().swap(r->w);
        std::vector<int32_t>().swap(r->layer);
      }
      char* ob = static_cast<char*>(s.out.p);
      clue_outputs out{reinterpret_cast<float*>(ob), reinterpret_cast<float*>(ob + 4 * pts),
                       reinterpret_cast<int32_t*>(ob + 8 * pts), reinterpret_cast<int32_t*>(ob + 12 * pts),
                       reinterpret_cast<int32_t*>(ob + 16 * pts)};
      Handle* h = reinterpret_cast<Handle*>(s.h);
      rc = h->run_batch(E, s.off.data(), reinterpret_cast<const float*>(ib),
                        reinterpret_cast<const float*>(ib + 4 * pts),
                        reinterpret_cast<const int32_t*>(ib + 8 * pts),
                        reinterpret_cast<const float*>(ib + 12 * pts), &out,
                        CLUE_HOST_MEMORY | CLUE_NO_GRAPH | kAsyncHostIO);
    }
    g.lock();
    if (rc) {
      for (Request* r : s.reqs) {
        r->status = rc;
        r->latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
      }
      s.reqs.clear();
      s.busy = false;
      done_cv_.notify_all();
      return true;
    }
    s.launched = true;
    ++batches_;
    batched_events_ += E;
    int inflight = 0;
    for (auto& t : slots_) inflight += t.busy;
    max_inflight_seen_ = std::max<double>(max_inflight_seen_, inflight);
    return true;
  }

  void loop() {
    cudaSetDevice(cfg_.device);
    std::unique_lock<std::mutex> g(mu_);
    while (!stop_) {
      reap(g);
      Slot* free_slot = nullptr;
      bool busy = false;
      for (auto& s : slots_) {
        if (!s.busy && !free_slot) free_slot = &s;
        busy |= s.busy;
      }
      if (free_slot && !queue_.empty()) {
        if (admit(*free_slot, g)) continue;
        // the head of the queue waits for device memory: a batch in flight
        // holds it, so look again once batches have been reaped
      }
      if (busy) {
        // batches in flight: look again shortly (new arrivals wake us earlier)
        cv_.wait_for(g, std::chrono::microseconds(20));
      } else {
        cv_.wait_for(g, std::chrono::milliseconds(5));
      }
    }
    // finish what is in flight before the slots are destroyed
    for (auto& s : slots_)
      if (s.launched) cudaEventSynchronize(reinterpret_cast<Handle*>(s.h)->done_event);
    reap(g);
    for (Request* r : queue_) r->status = CLUE_EINVAL;
    queue_.clear();
    done_cv_.notify_all();
  }

  clue_params params_;
  clue_server_config cfg_;
  std::vector<Slot> slots_;
  size_t budget_ = 0;
  int64_t cap_points_ = 0;
  int64_t memory_waits_ = 0;
  int64_t waiting_id_ = 0;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> queue_;
  std::unordered_map<int64_t, Request*> reqs_;
  int64_t next_id_ = 1;
  bool stop_ = false;
  std::thread worker_;
  CopyPool pool_;  // its helpers stop when the server is destroyed, after shutdown() joined worker_
  std::vector<double> lat_;
  int64_t batches_ = 0, batched_events_ = 0;
  double max_inflight_seen_ = 0;
};

}  // namespace
}  // namespace clue

using clue::Server;
using clue::set_error;

extern "C" {

int clue_server_create(const clue_params* params, const clue_server_config* cfg, clue_server** out) {
  return clue::guarded([&]() -> int {
    if (!params || !cfg || !out) return set_error(CLUE_EINVAL, "NULL argument");
    *out = nullptr;
    Server* s = new Server(*params, *cfg);
    int rc = s->start();
    if (rc) {
      delete s;
      return rc;
    }
    *out = reinterpret_cast<clue_server*>(s);
    return CLUE_OK;
  });
}

int clue_server_destroy(clue_server* s) {
  delete reinterpret_cast<Server*>(s);
  return CLUE_OK;
}

int clue_server_submit(clue_server* s, int32_t n, const float* x, const float* y, const int32_t* layer,
                       const float* weight, const clue_outputs* out, int64_t* request_id) {
  return clue::guarded([&]() -> int {
    if (!s) return set_error(CLUE_EINVAL, "NULL server");
    return reinterpret_cast<Server*>(s)->submit(n, x, y, layer, weight, out, request_id);
  });
}

int clue_server_submit_many(clue_server* s, int32_t n_events, const int64_t* event_offsets, const float* x,
                            const float* y, const int32_t* layer, const float* weight, const clue_outputs* outs,
                            int64_t* request_ids) {
  return clue::guarded([&]() -> int {
    if (!s) return set_error(CLUE_EINVAL, "NULL server");
    return reinterpret_cast<Server*>(s)->submit_many(n_events, event_offsets, x, y, layer, weight, outs, request_ids);
  });
}

int clue_server_poll(clue_server* s, int64_t id, int32_t timeout_ms, double* latency_ms) {
  return clue::guarded([&]() -> int {
    if (!s) return set_error(CLUE_EINVAL, "NULL server");
    return reinterpret_cast<Server*>(s)->poll(id, timeout_ms, latency_ms);
  });
}

int clue_server_drain(clue_server* s, int32_t timeout_ms) {
  return clue::guarded([&]() -> int {
    if (!s) return set_error(CLUE_EINVAL, "NULL server");
    return reinterpret_cast<Server*>(s)->drain(timeout_ms);
  });
}

int clue_server_get_stats(clue_server* s, clue_server_stats* st) {
  return clue::guarded([&]() -> int {
    if (!s || !st) return set_error(CLUE_EINVAL, "NULL argument");
    reinterpret_cast<Server*>(s)->stats(st);
    return CLUE_OK;
  });
}

int clue_server_reset_stats(clue_server* s) {
  if (!s) return set_error(CLUE_EINVAL, "NULL server");
  reinterpret_cast<Server*>(s)->reset_stats();
  return CLUE_OK;
}

}  // extern "C"
