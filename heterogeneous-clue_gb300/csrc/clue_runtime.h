// Host-side runtime objects behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <exception>
#include <new>
#include <cstdint>
#include <vector>

#include "../../include/clue.h"
#include "clue_internal.h"

namespace clue {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

// Runs f() and turns a C++ exception into a status code: nothing may unwind
// through the C ABI (a host allocation failing is CLUE_ENOMEM).
template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return set_error(CLUE_ENOMEM, "host memory allocation failed");
  } catch (const std::exception& e) {
    return set_error(CLUE_EINVAL, "internal error: %s", e.what());
  } catch (...) {
    return set_error(CLUE_EINVAL, "internal error");
  }
}

// Named, grow-only device buffers under a byte budget.  Buffers are only
// reallocated when a request outgrows them, never per call.
class DeviceArena {
 public:
  ~DeviceArena();
  int reserve(const std::vector<size_t>& need, size_t budget);
  // Device bytes the arena would hold after reserve(need) without the growth
  // margin (the margin is only taken when the budget has room for it).
  size_t bytes_after(const std::vector<size_t>& need) const;
  void* ptr(int slot) const { return slot < (int)bufs_.size() ? bufs_[slot].p : nullptr; }
  size_t total() const { return total_; }
  uint64_t generation() const { return gen_; }  // bumped whenever a buffer is (re)allocated
  void release();

 private:
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  std::vector<Buf> bufs_;
  size_t total_ = 0;
  uint64_t gen_ = 0;
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~PinnedBuf();
  int reserve(size_t n);
};

// Everything a captured 2D graph bakes in.
struct GraphKey {
  int32_t E = -1;
  int64_t N = -1;
  int64_t nchunks = -1;     // launch sizes of the chunk kernels are baked into the graph
  uint64_t arena_gen = 0;   // and so are the addresses of every arena buffer
  int flags = 0;
  int threads = 0, cap = 0, ctas = 0, big_threads = 0, big_cap = 0;
  float work_tile = 0.f;
  float dc = 0.f, rhoc = 0.f, odf = 0.f;
  const void* ptrs[14] = {};
  bool operator==(const GraphKey& o) const {
    if (E != o.E || N != o.N || nchunks != o.nchunks || arena_gen != o.arena_gen || flags != o.flags ||
        threads != o.threads || cap != o.cap || ctas != o.ctas ||
        big_threads != o.big_threads || big_cap != o.big_cap ||
        work_tile != o.work_tile || dc != o.dc || rhoc != o.rhoc || odf != o.odf)
      return false;
    for (int i = 0; i < 14; ++i)
      if (ptrs[i] != o.ptrs[i]) return false;
    return true;
  }
};

size_t required_bytes_2d(int32_t E, int64_t N, int64_t nchunks, int grid, bool host_io);
struct Handle;
// Sizes the handle's 2D buffers for a batch of E events and N points ahead of
// time (a server slot does this at start so that its first batches do not
// allocate).
int reserve_2d(Handle* h, int32_t E, int64_t N, bool host_io);
// Device bytes the handle's 2D arena would hold after sizing it for a batch of
// E events, N points and nchunks chunks (the batch's own chunk count).
size_t arena_bytes_after_2d(const Handle* h, int32_t E, int64_t N, int64_t nchunks, bool host_io);

// Internal run flag: host (pinned) buffers, but return once the work is
// queued; completion is seen through Handle::done_event.  Used by the server.
constexpr int kAsyncHostIO = 0x100;

// Device slots of the pipelined host-memory path (sub-batches in flight).
constexpr int kPipeSlots = 2;

struct Handle {
  int device = 0;
  size_t budget = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t owned_stream = nullptr;  // created by the handle, destroyed with it
  cudaEvent_t done_event = nullptr;
  bool pending = false;
  int error_layers = kLayers;
  Params2D p2d{};
  Tuning2D tuning{};
  DeviceArena arena;
  DeviceArena arena3d;
  DeviceArena arena_bridge;
  DeviceArena arena_pipe[kPipeSlots - 1];  // further slots of the pipelined host-memory path
  cudaStream_t copy_in = nullptr;         // pipelined host-memory path: H2D stream
  cudaStream_t copy_out = nullptr;        // and D2H stream
  cudaEvent_t pipe_events[3 * kPipeSlots] = {};  // per slot: H2D done, kernels done, D2H done
  clue_run_stats last_run{};              // copies and kernels of the last 2D run
  int64_t graph_kernels = 0;              // kernels in graph_exec
  PinnedBuf stage;
  PinnedBuf flags_host;
  PinnedBuf nt_host;
  cudaGraphExec_t graph_exec = nullptr;
  GraphKey graph_key;
  GraphKey last_key;  // the previous graph-eligible run (a shape is captured when it repeats)

  ~Handle();
  int wait_previous();
  int check_device_flags();
  int profile_batch(int32_t E, const int64_t* off, const float* x, const float* y, const int32_t* layer,
                    const float* w, const clue_outputs* out, float* stage_ms);
  int run_batch(int32_t E, const int64_t* off, const float* x, const float* y, const int32_t* layer, const float* w,
                const clue_outputs* out, int flags);
};

}  // namespace clue
