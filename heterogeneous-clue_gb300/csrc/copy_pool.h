// Resident host-copy pool (host-only C++, no CUDA).
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

namespace clue {

// Host copies of the serving path (request staging and result delivery) and
// the host passes of the pipelined host-memory path.  Work is cut into
// pieces shared by the calling thread and resident helper threads (no thread
// is started per call): copy sets of 512 KB or more in 256 KB pieces, or a
// caller's own function over numbered pieces (for_pieces).  Several callers
// (submitting clients, the scheduler) may run sets at once: a helper takes at
// most four pieces of a set before it moves on to the next set, so that no
// set waits behind a large one.
struct CopyTask {
  void* dst;
  const void* src;
  size_t bytes;
};

class CopyPool {
 public:
  ~CopyPool() { stop(); }

  void start(int helpers) {
    for (int k = 0; k < helpers; ++k) {
      try {
        threads_.emplace_back([this] { loop(); });
      } catch (...) {
        break;  // fewer helpers: callers do their own pieces
      }
    }
  }
  bool started() const { return !threads_.empty(); }

  void stop() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
    threads_.clear();
  }

  void run(const std::vector<CopyTask>& tasks) {
    constexpr size_t kPiece = size_t(256) << 10;
    size_t total = 0;
    for (const auto& t : tasks) total += t.bytes;
    if (threads_.empty() || total < 2 * kPiece) {
      for (const auto& t : tasks)
        if (t.bytes) memcpy(t.dst, t.src, t.bytes);
      return;
    }
    std::vector<CopyTask> pieces;
    for (const auto& t : tasks)
      for (size_t o = 0; o < t.bytes; o += kPiece)
        pieces.push_back({static_cast<char*>(t.dst) + o, static_cast<const char*>(t.src) + o,
                          std::min(kPiece, t.bytes - o)});
    for_pieces(pieces.size(), [&](size_t i) { memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes); });
  }

  // Calls f(0) .. f(n - 1), each once, on the calling thread and the helpers;
  // returns when all calls have returned.
  template <class F>
  void for_pieces(size_t n, F&& f) {
    if (n == 0) return;
    if (threads_.empty() || n == 1) {
      for (size_t i = 0; i < n; ++i) f(i);
      return;
    }
    Job job;
    job.n = n;
    job.fn = [](void* ctx, size_t i) { (*static_cast<F*>(ctx))(i); };
    job.ctx = &f;
    job.left = n;
    {
      std::lock_guard<std::mutex> g(mu_);
      jobs_.push_back(&job);
    }
    cv_.notify_all();
    work(job);
    // the job lives on this stack: wait until no helper holds it any more
    std::unique_lock<std::mutex> g(mu_);
    done_cv_.wait(g, [&] { return job.left.load() == 0 && job.holders == 0; });
    auto it = std::find(jobs_.begin(), jobs_.end(), &job);
    if (it != jobs_.end()) jobs_.erase(it);
  }

 private:
  struct Job {
    size_t n = 0;
    void (*fn)(void*, size_t) = nullptr;
    void* ctx = nullptr;
    std::atomic<size_t> next{0};
    std::atomic<size_t> left{0};
    int holders = 0;  // helpers working on it (guarded by mu_)
  };

  static void work(Job& j, size_t max_pieces = SIZE_MAX) {
    for (size_t i, k = 0; k < max_pieces && (i = j.next.fetch_add(1)) < j.n; ++k) {
      j.fn(j.ctx, i);
      j.left.fetch_sub(1);
    }
  }

  void loop() {
    std::unique_lock<std::mutex> g(mu_);
    for (;;) {
      cv_.wait(g, [&] { return stop_ || !jobs_.empty(); });
      if (stop_) return;
      Job* j = jobs_.front();
      jobs_.pop_front();
      if (j->next.load() >= j->n) {  // nothing left to take: let the owner finish it
        done_cv_.notify_all();
        continue;
      }
      jobs_.push_back(j);  // round robin over the sets in progress
      ++j->holders;
      g.unlock();
      work(*j, 4);
      g.lock();
      --j->holders;
      done_cv_.notify_all();
    }
  }

  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Job*> jobs_;
  bool stop_ = false;
};

}  // namespace clue
