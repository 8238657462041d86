// Host runtime and C ABI of the CLUE path: handles, resident device arena,
// batch planning, CUDA-graph replay and error reporting.
//
// Replaces, for the clusterizer path only, the reference's per-event
// CLUEAlgoCUDA object (src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.{h,cu}):
// there the algorithm owns fixed tile/follower scratch and allocates a
// PointsCloudCUDA per event from the caching allocator; here a handle owns
// grow-only device buffers sized for the largest batch seen, capped by a
// budget, and nothing is allocated on the steady-state path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/clue.h"
#include "clue_internal.h"
#include "clue_runtime.h"

static_assert(clue::kStages2D == CLUE_N_STAGES, "stage list of the ABI and of the pipeline differ");

namespace clue {

thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear sticky-free errors so the next call starts clean
  return set_error(CLUE_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// ------------------------------------------------------------------ Arena --

DeviceArena::~DeviceArena() { release(); }

void DeviceArena::release() {
  for (auto& b : bufs_) {
    if (b.p) cudaFree(b.p);
    b = Buf{};
  }
  total_ = 0;
  ++gen_;
}

int DeviceArena::reserve(const std::vector<size_t>& need_in, size_t budget) {
  // A buffer that must grow grows by at least half its size when the budget
  // allows, so that slowly rising request sizes do not reallocate every call.
  std::vector<size_t> need = need_in;
  size_t want = 0, want_grown = 0;
  for (size_t i = 0; i < need.size(); ++i) {
    const size_t have = i < bufs_.size() ? bufs_[i].bytes : 0;
    want += std::max(need[i], have);
    want_grown += need[i] <= have ? have : std::max(need[i], have + have / 2);
  }
  if (want > budget)
    return set_error(CLUE_ENOMEM, "request needs %zu device bytes, budget is %zu", want, budget);
  if (want_grown <= budget)
    for (size_t i = 0; i < need.size(); ++i) {
      const size_t have = i < bufs_.size() ? bufs_[i].bytes : 0;
      if (need[i] > have) need[i] = std::max(need[i], have + have / 2);
    }
  if (bufs_.size() < need.size()) bufs_.resize(need.size());
  for (size_t i = 0; i < need.size(); ++i) {
    if (need[i] <= bufs_[i].bytes) continue;
    if (bufs_[i].p) {
      cudaFree(bufs_[i].p);
      total_ -= bufs_[i].bytes;
      bufs_[i] = Buf{};
    }
    size_t bytes = (need[i] + 255) & ~size_t(255);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(CLUE_ENOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    bufs_[i].p = p;
    bufs_[i].bytes = bytes;
    total_ += bytes;
    ++gen_;
  }
  return CLUE_OK;
}

size_t DeviceArena::bytes_after(const std::vector<size_t>& need) const {
  size_t t = 0;
  for (size_t i = 0; i < need.size(); ++i) {
    const size_t have = i < bufs_.size() ? bufs_[i].bytes : 0;
    t += std::max((need[i] + 255) & ~size_t(255), have);
  }
  for (size_t i = need.size(); i < bufs_.size(); ++i) t += bufs_[i].bytes;
  return t;
}

PinnedBuf::~PinnedBuf() {
  if (p) cudaFreeHost(p);
}

int PinnedBuf::reserve(size_t n) {
  if (n <= bytes) return CLUE_OK;
  const size_t b = std::max<size_t>({n, size_t(4096), bytes + bytes / 2});
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
  cudaError_t e = cudaHostAlloc(&p, b, cudaHostAllocDefault);
  if (e != cudaSuccess) return cuda_error(e, "cudaHostAlloc");
  bytes = b;
  return CLUE_OK;
}

// ------------------------------------------------------------ 2D planning --

namespace {

enum Slot2D : int {
  S_OFF, S_CS, S_LCNT, S_LSTART, S_CURSOR, S_GX, S_GY, S_GW, S_GID,
  S_SP0, S_SP1, S_SP2, S_SP3, S_SP4, S_SP5, S_SP6, S_SP7,
  S_SPTBL, S_CSEED, S_CBASE, S_FLAGS, S_ORDER, S_CEV,
  S_IN,   // host runs: x | y | layer | w of the run, each N long, back to back
  S_OUT,  // host runs: rho | delta | nearestHigher | isSeed | clusterIndex, likewise
  S_COUNT
};

int64_t n_chunks_of(int32_t n_events, const int64_t* off) {
  int64_t c = 0;
  for (int32_t e = 0; e < n_events; ++e) c += (off[e + 1] - off[e] + kChunk - 1) / kChunk;
  return c;
}

std::vector<size_t> sizes_2d(int32_t E, int64_t N, int64_t nchunks, int grid, bool host_io) {
  std::vector<size_t> s(S_COUNT, 0);
  s[S_OFF] = 8 * (size_t)(E + 1);
  s[S_CS] = 4 * (size_t)(E + 1);
  s[S_LCNT] = s[S_LSTART] = s[S_CURSOR] = 4 * (size_t)E * kLayers;
  s[S_GX] = s[S_GY] = s[S_GW] = s[S_GID] = 4 * (size_t)N;
  // spill homes: 16-byte records, then nh and the query order (4 B each)
  s[S_SP0] = 16 * (size_t)N;
  s[S_SP1] = s[S_SP2] = s[S_SP3] = s[S_SP6] = s[S_SP7] = 0;
  s[S_SP4] = s[S_SP5] = 4 * (size_t)N;
  s[S_SPTBL] = 4 * (size_t)kTableStride * grid;
  s[S_CSEED] = s[S_CBASE] = s[S_CEV] = 4 * (size_t)std::max<int64_t>(nchunks, 1);
  s[S_FLAGS] = 4 * kFlagCount;
  s[S_ORDER] = 4 * ((size_t)E * kLayers + 2 * kSizeBuckets);
  if (host_io) {
    s[S_IN] = 16 * (size_t)N;
    s[S_OUT] = 20 * (size_t)N;
  }
  return s;
}

bool is_pinned_or_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

size_t required_bytes_2d(int32_t E, int64_t N, int64_t nchunks, int grid, bool host_io) {
  auto s = sizes_2d(E, N, nchunks, grid, host_io);
  size_t t = 0;
  for (size_t v : s) t += (v + 255) & ~size_t(255);
  return t;
}

int reserve_2d(Handle* h, int32_t E, int64_t N, bool host_io) {
  const int64_t nchunks = N / kChunk + E;
  const int grid = layer_grid_max(h->tuning, std::max(1, E * kLayers));
  int rc = h->arena.reserve(sizes_2d(E, N, nchunks, grid, host_io), h->budget);
  if (!rc) rc = h->stage.reserve(24 * (size_t)(E + 1) + 4 * (size_t)nchunks);
  if (!rc) rc = h->flags_host.reserve(4 * kFlagCount);
  return rc;
}

size_t arena_bytes_after_2d(const Handle* h, int32_t E, int64_t N, int64_t nchunks, bool host_io) {
  const int grid = layer_grid_max(h->tuning, std::max(1, E * kLayers));
  return h->arena.bytes_after(sizes_2d(E, N, nchunks, grid, host_io));
}

Handle::~Handle() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (done_event) cudaEventDestroy(done_event);
  for (auto ev : pipe_events)
    if (ev) cudaEventDestroy(ev);
  if (copy_in) cudaStreamDestroy(copy_in);
  if (copy_out) cudaStreamDestroy(copy_out);
  arena.release();
  if (owned_stream) cudaStreamDestroy(owned_stream);
}

int Handle::wait_previous() {
  if (!pending) return CLUE_OK;
  cudaError_t e = cudaEventSynchronize(done_event);
  pending = false;
  if (e != cudaSuccess) return cuda_error(e, "waiting for previous run");
  return CLUE_OK;
}

int Handle::check_device_flags() {
  const int32_t* f = static_cast<const int32_t*>(flags_host.p);
  if (f && f[kFlagError]) {
    const_cast<int32_t*>(f)[kFlagError] = 0;
    return set_error(CLUE_EINVAL, "a point has a layer outside [0, %d)", error_layers ? error_layers : kLayers);
  }
  return CLUE_OK;
}

namespace {

struct Run2D {
  int32_t E;
  int64_t N;
  const int64_t* off;  // host
  const float* x;
  const float* y;
  const int32_t* layer;
  const float* w;
  const clue_outputs* out;
  int flags;
};

int validate_offsets(int32_t E, const int64_t* off) {
  if (E < 0) return set_error(CLUE_EINVAL, "n_events < 0");
  if (E == 0) return CLUE_OK;
  if (!off) return set_error(CLUE_EINVAL, "event_offsets is NULL");
  if (off[0] != 0) return set_error(CLUE_EINVAL, "event_offsets[0] must be 0");
  for (int32_t e = 0; e < E; ++e)
    if (off[e + 1] < off[e]) return set_error(CLUE_EINVAL, "event_offsets must be non-decreasing");
  if (off[E] > INT32_MAX) return set_error(CLUE_EINVAL, "more than 2^31-1 points in one call");
  return CLUE_OK;
}

// Queues the batch pipeline (copies included in host mode) on h->stream.
int enqueue_2d(Handle* h, const Run2D& r, Batch2D& b, bool host_io, cudaEvent_t* stage_events = nullptr,
               int64_t* kernels = nullptr) {
  cudaStream_t s = h->stream;
  cudaError_t e;
  const size_t n4 = 4 * (size_t)r.N;
  e = cudaMemsetAsync(b.flags + kFlagError, 0, 4, s);
  if (e != cudaSuccess) return cuda_error(e, "clearing status");
  e = cudaMemcpyAsync((void*)b.offsets, h->stage.p, 8 * (size_t)(r.E + 1), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "H2D offsets");
  e = cudaMemcpyAsync((void*)b.chunk_start, static_cast<char*>(h->stage.p) + 8 * (size_t)(r.E + 1),
                      4 * (size_t)(r.E + 1), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "H2D chunk table");
  e = cudaMemcpyAsync((void*)b.chunk_ev, static_cast<char*>(h->stage.p) + 12 * (size_t)(r.E + 1),
                      4 * (size_t)b.n_chunks, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "H2D chunk events");
  if (host_io) {
    // back-to-back host arrays (a server's staging) move in one copy
    const char* hx = reinterpret_cast<const char*>(r.x);
    if (reinterpret_cast<const char*>(r.y) == hx + n4 && reinterpret_cast<const char*>(r.layer) == hx + 2 * n4 &&
        reinterpret_cast<const char*>(r.w) == hx + 3 * n4) {
      if ((e = cudaMemcpyAsync((void*)b.x, r.x, 4 * n4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_error(e, "H2D points");
    } else if ((e = cudaMemcpyAsync((void*)b.x, r.x, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync((void*)b.y, r.y, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync((void*)b.layer, r.layer, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync((void*)b.w, r.w, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess) {
      return cuda_error(e, "H2D points");
    }
  }
  e = launch_clue2d(b, h->p2d, h->tuning, s, stage_events, kernels);
  if (e != cudaSuccess) return cuda_error(e, "launching CLUE kernels");
  if (host_io) {
    const clue_outputs* o = r.out;
    const char* ho = reinterpret_cast<const char*>(o->rho);
    if (reinterpret_cast<const char*>(o->delta) == ho + n4 &&
        reinterpret_cast<const char*>(o->nearestHigher) == ho + 2 * n4 &&
        reinterpret_cast<const char*>(o->isSeed) == ho + 3 * n4 &&
        reinterpret_cast<const char*>(o->clusterIndex) == ho + 4 * n4) {
      if ((e = cudaMemcpyAsync(o->rho, b.rho, 5 * n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_error(e, "D2H outputs");
    } else if ((e = cudaMemcpyAsync(o->rho, b.rho, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(o->delta, b.delta, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(o->nearestHigher, b.nh, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(o->isSeed, b.seed, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(o->clusterIndex, b.ci, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
      return cuda_error(e, "D2H outputs");
    }
  }
  e = cudaMemcpyAsync(h->flags_host.p, b.flags, 4 * kFlagCount, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_error(e, "D2H status");
  return CLUE_OK;
}

// Device inputs and outputs of a host-memory run of N points: each array N
// long, back to back, so that back-to-back host arrays move in one copy.
void host_io_views(void* in, void* out, int64_t N, Batch2D& b) {
  float* fi = static_cast<float*>(in);
  float* fo = static_cast<float*>(out);
  b.x = fi;
  b.y = fi + N;
  b.layer = reinterpret_cast<const int32_t*>(fi + 2 * N);
  b.w = fi + 3 * N;
  b.rho = fo;
  b.delta = fo + N;
  b.nh = reinterpret_cast<int32_t*>(fo + 2 * N);
  b.seed = reinterpret_cast<int32_t*>(fo + 3 * N);
  b.ci = reinterpret_cast<int32_t*>(fo + 4 * N);
}

void fill_batch_views(Handle* h, const Run2D& r, int64_t nchunks, bool host_io, Batch2D& b,
                      const DeviceArena* arena = nullptr) {
  const DeviceArena& A = arena ? *arena : h->arena;
  auto P = [&](int slot) { return A.ptr(slot); };
  b.n_events = r.E;
  b.n_points = r.N;
  b.n_chunks = (int32_t)nchunks;
  b.offsets = static_cast<const int64_t*>(P(S_OFF));
  b.chunk_start = static_cast<const int32_t*>(P(S_CS));
  if (host_io) {
    host_io_views(P(S_IN), P(S_OUT), r.N, b);
  } else {
    b.x = r.x;
    b.y = r.y;
    b.layer = r.layer;
    b.w = r.w;
    b.rho = r.out->rho;
    b.delta = r.out->delta;
    b.nh = r.out->nearestHigher;
    b.seed = r.out->isSeed;
    b.ci = r.out->clusterIndex;
  }
  b.lcnt = static_cast<int32_t*>(P(S_LCNT));
  b.lstart = static_cast<int32_t*>(P(S_LSTART));
  b.cursor = static_cast<int32_t*>(P(S_CURSOR));
  b.gx = static_cast<float*>(P(S_GX));
  b.gy = static_cast<float*>(P(S_GY));
  b.gw = static_cast<float*>(P(S_GW));
  b.gid = static_cast<int32_t*>(P(S_GID));
  for (int i = 0; i < 8; ++i) b.sp[i] = static_cast<float*>(P(S_SP0 + i));
  b.sp_tbl = static_cast<int32_t*>(P(S_SPTBL));
  b.chunk_seeds = static_cast<int32_t*>(P(S_CSEED));
  b.chunk_base = static_cast<int32_t*>(P(S_CBASE));
  b.chunk_ev = static_cast<const int32_t*>(P(S_CEV));
  b.flags = static_cast<int32_t*>(P(S_FLAGS));
  b.order = static_cast<int32_t*>(P(S_ORDER));
  b.size_hist = b.order + (size_t)r.E * kLayers;
}

int run_2d_batched(Handle* h, const Run2D& r, cudaEvent_t* stage_events = nullptr) {
  const bool host_io = !(r.flags & CLUE_DEVICE_MEMORY);
  int rc = h->wait_previous();
  if (rc) return rc;
  const int64_t nchunks = n_chunks_of(r.E, r.off);
  const int grid = layer_grid_max(h->tuning, std::max(1, r.E * kLayers));
  rc = h->arena.reserve(sizes_2d(r.E, r.N, nchunks, grid, host_io), h->budget);
  if (rc) return rc;
  // offsets + chunk table through pinned staging (graph nodes copy from it)
  rc = h->stage.reserve(12 * (size_t)(r.E + 1) + 4 * (size_t)nchunks);
  if (rc) return rc;
  int64_t* so = static_cast<int64_t*>(h->stage.p);
  int32_t* sc = reinterpret_cast<int32_t*>(static_cast<char*>(h->stage.p) + 8 * (size_t)(r.E + 1));
  int32_t* sce = sc + (r.E + 1);  // event of each chunk
  memcpy(so, r.off, 8 * (size_t)(r.E + 1));
  sc[0] = 0;
  for (int32_t e = 0; e < r.E; ++e) {
    sc[e + 1] = sc[e] + (int32_t)((r.off[e + 1] - r.off[e] + kChunk - 1) / kChunk);
    for (int32_t c = sc[e]; c < sc[e + 1]; ++c) sce[c] = e;
  }
  rc = h->flags_host.reserve(4 * kFlagCount);
  if (rc) return rc;

  Batch2D b;
  fill_batch_views(h, r, nchunks, host_io, b);

  bool use_graph = !(r.flags & CLUE_NO_GRAPH) && !stage_events;
  if (use_graph && host_io) {
    // graph memcpy nodes need page-locked host memory
    use_graph = is_pinned_or_device(r.x) && is_pinned_or_device(r.y) && is_pinned_or_device(r.layer) &&
                is_pinned_or_device(r.w) && is_pinned_or_device(r.out->rho) &&
                is_pinned_or_device(r.out->delta) && is_pinned_or_device(r.out->nearestHigher) &&
                is_pinned_or_device(r.out->isSeed) && is_pinned_or_device(r.out->clusterIndex);
  }
  cudaError_t e;
  int64_t kernels = 0;
  if (use_graph) {
    GraphKey key{r.E, r.N, nchunks, h->arena.generation(), r.flags, h->tuning.threads, h->tuning.layer_capacity,
                 h->tuning.ctas_per_sm,
                 h->tuning.big_threads, h->tuning.big_capacity,
                 h->tuning.work_tile_cm, h->p2d.dc, h->p2d.rhoc, h->p2d.odf,
                 {(const void*)r.x, (const void*)r.y, (const void*)r.layer, (const void*)r.w,
                  (const void*)r.out->rho, (const void*)r.out->delta, (const void*)r.out->nearestHigher,
                  (const void*)r.out->isSeed, (const void*)r.out->clusterIndex, h->arena.ptr(S_OFF),
                  h->arena.ptr(S_GX), h->arena.ptr(S_SP0), h->stage.p, h->flags_host.p}};
    // A graph pays off when a shape repeats (the same event sizes, buffers and
    // tuning): a run whose key differs from the previous run's goes by direct
    // launches, and the second run in a row with one key is captured and
    // replayed from then on.  A producer that sees a new event size on every
    // call never pays for a capture (measured: 0.181 ms per 50k-150k-point
    // event with a capture per call, 0.129 ms direct, 0.100 ms replayed).
    const bool repeated = key == h->last_key;
    h->last_key = key;
    use_graph = (h->graph_exec && key == h->graph_key) || repeated;
  }
  if (use_graph) {
    const GraphKey& key = h->last_key;
    if (!h->graph_exec || !(key == h->graph_key)) {
      if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
      }
      cudaStream_t s = h->stream;
      e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return cuda_error(e, "cudaStreamBeginCapture");
      h->graph_kernels = 0;
      rc = enqueue_2d(h, r, b, host_io, nullptr, &h->graph_kernels);
      cudaGraph_t g = nullptr;
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        h->graph_kernels = 0;
        return rc;
      }
      if (e2 != cudaSuccess) return cuda_error(e2, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&h->graph_exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        h->graph_exec = nullptr;
        return cuda_error(e, "cudaGraphInstantiate");
      }
      h->graph_key = key;
    }
    NvtxRange nr("clue2d/graph_replay");
    e = cudaGraphLaunch(h->graph_exec, h->stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
    kernels = h->graph_kernels;
  } else {
    rc = enqueue_2d(h, r, b, host_io, stage_events, &kernels);
    if (rc) return rc;
  }
  e = cudaEventRecord(h->done_event, h->stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaEventRecord");
  h->pending = true;
  h->error_layers = kLayers;
  h->last_run.h2d_bytes = 12 * (int64_t)(r.E + 1) + 4 * nchunks + (host_io ? 16 * r.N : 0);
  h->last_run.d2h_bytes = 4 * kFlagCount + (host_io ? 20 * r.N : 0);
  h->last_run.kernel_launches = kernels;
  if (host_io && !(r.flags & kAsyncHostIO)) {
    rc = h->wait_previous();
    if (rc) return rc;
    return h->check_device_flags();
  }
  return CLUE_OK;
}

// The plain form: one event per launch sequence, the same kernels.
int run_2d_plain(Handle* h, const Run2D& r) {
  const bool host_io = !(r.flags & CLUE_DEVICE_MEMORY);
  int rc = h->wait_previous();
  if (rc) return rc;
  int64_t maxn = 0;
  for (int32_t e = 0; e < r.E; ++e) maxn = std::max(maxn, r.off[e + 1] - r.off[e]);
  const int64_t maxchunks = (maxn + kChunk - 1) / kChunk;
  const int grid = layer_grid_max(h->tuning, kLayers);
  auto need = sizes_2d(1, maxn, maxchunks, grid, false);
  if (host_io) {
    need[S_IN] = 16 * (size_t)maxn;
    need[S_OUT] = 20 * (size_t)maxn;
  }
  need[S_OFF] = 16 * (size_t)std::max(r.E, 1);
  need[S_CS] = 8 * (size_t)std::max(r.E, 1);
  rc = h->arena.reserve(need, h->budget);
  if (rc) return rc;
  rc = h->stage.reserve(24 * (size_t)std::max(r.E, 1));
  if (rc) return rc;
  rc = h->flags_host.reserve(4 * kFlagCount);
  if (rc) return rc;
  int64_t* so = static_cast<int64_t*>(h->stage.p);
  int32_t* sc = reinterpret_cast<int32_t*>(so + 2 * (size_t)r.E);
  for (int32_t e = 0; e < r.E; ++e) {
    so[2 * e] = 0;
    so[2 * e + 1] = r.off[e + 1] - r.off[e];
    sc[2 * e] = 0;
    sc[2 * e + 1] = (int32_t)((so[2 * e + 1] + kChunk - 1) / kChunk);
  }
  cudaStream_t s = h->stream;
  cudaError_t e = cudaMemsetAsync(h->arena.ptr(S_FLAGS), 0, 4 * kFlagCount, s);
  if (e != cudaSuccess) return cuda_error(e, "clearing status");
  e = cudaMemcpyAsync(h->arena.ptr(S_OFF), so, 16 * (size_t)r.E, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "H2D offsets");
  e = cudaMemcpyAsync(h->arena.ptr(S_CS), sc, 8 * (size_t)r.E, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "H2D chunk table");
  int any_error = 0;
  h->last_run.h2d_bytes = 24 * (int64_t)r.E + (host_io ? 16 * r.N : 0);
  h->last_run.d2h_bytes = 0;
  h->last_run.kernel_launches = 0;
  for (int32_t ev = 0; ev < r.E; ++ev) {
    const int64_t s0 = r.off[ev], n = r.off[ev + 1] - s0;
    if (n == 0) continue;
    Run2D one = r;
    one.E = 1;
    one.N = n;
    Batch2D b;
    fill_batch_views(h, one, sc[2 * ev + 1], false, b);
    b.chunk_ev = nullptr;  // one event: every chunk is event 0
    b.offsets = static_cast<const int64_t*>(h->arena.ptr(S_OFF)) + 2 * ev;
    b.chunk_start = static_cast<const int32_t*>(h->arena.ptr(S_CS)) + 2 * ev;
    const size_t n4 = 4 * (size_t)n;
    if (host_io) {
      host_io_views(h->arena.ptr(S_IN), h->arena.ptr(S_OUT), n, b);
      if ((e = cudaMemcpyAsync((void*)b.x, r.x + s0, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync((void*)b.y, r.y + s0, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync((void*)b.layer, r.layer + s0, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync((void*)b.w, r.w + s0, n4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_error(e, "H2D points");
    } else {
      b.x = r.x + s0;
      b.y = r.y + s0;
      b.layer = r.layer + s0;
      b.w = r.w + s0;
      b.rho = r.out->rho + s0;
      b.delta = r.out->delta + s0;
      b.nh = r.out->nearestHigher + s0;
      b.seed = r.out->isSeed + s0;
      b.ci = r.out->clusterIndex + s0;
    }
    e = launch_clue2d(b, h->p2d, h->tuning, s, nullptr, &h->last_run.kernel_launches);
    if (e != cudaSuccess) return cuda_error(e, "launching CLUE kernels");
    if (host_io) {
      const clue_outputs* o = r.out;
      if ((e = cudaMemcpyAsync(o->rho + s0, b.rho, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(o->delta + s0, b.delta, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(o->nearestHigher + s0, b.nh, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(o->isSeed + s0, b.seed, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(o->clusterIndex + s0, b.ci, n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_error(e, "D2H outputs");
      // the reference's CUDA producer synchronises per event (CLUEAlgoCUDA.cu:80)
      e = cudaMemcpyAsync(h->flags_host.p, b.flags, 4 * kFlagCount, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_error(e, "per-event synchronise");
      any_error |= static_cast<int32_t*>(h->flags_host.p)[kFlagError];
      h->last_run.d2h_bytes += 20 * n + 4 * kFlagCount;
    }
  }
  if (host_io) {
    if (any_error) return set_error(CLUE_EINVAL, "a point has a layer outside [0, %d)", kLayers);
    return CLUE_OK;
  }
  // device mode: the error word accumulates over the events (launch_clue2d
  // never clears it) and is read back at clue_synchronize.
  e = cudaMemcpyAsync(h->flags_host.p, h->arena.ptr(S_FLAGS), 4 * kFlagCount, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_error(e, "D2H status");
  h->last_run.d2h_bytes = 4 * kFlagCount;
  e = cudaEventRecord(h->done_event, s);
  if (e != cudaSuccess) return cuda_error(e, "cudaEventRecord");
  h->pending = true;
  h->error_layers = kLayers;
  return CLUE_OK;
}

// Host-memory batches of at least 2 * kPipePoints points: the events are cut
// into sub-batches of about kPipePoints points that take turns on
// kPipeSlots device slots.  Three streams overlap the H2D copy of one sub-batch, the
// kernels of the previous one and the D2H copy of the one before that:
//   in-copy  : wait comp[k] (slot inputs free)  -> offsets, chunk table, x, y, layer, w -> h2d[k]
//   compute  : wait h2d[k], d2h[k] (slot outputs free) -> kernels -> comp[k]
//   out-copy : wait comp[k] -> rho, delta, nh, isSeed, clusterIndex, status -> d2h[k]
// Sub-batches hold whole events, so every output is the one of the
// unsplit batch.
constexpr int64_t kPipePoints = int64_t(8) << 20;

int run_2d_pipelined(Handle* h, const Run2D& r) {
  int rc = h->wait_previous();
  if (rc) return rc;
  // event-aligned cuts
  std::vector<int32_t> cut{0};
  for (int32_t e = 0; e < r.E; ++e)
    if (r.off[e + 1] - r.off[cut.back()] >= kPipePoints && e + 1 < r.E) cut.push_back(e + 1);
  cut.push_back(r.E);
  const int S = (int)cut.size() - 1;
  int32_t maxE = 0;
  int64_t maxN = 0, maxC = 0;
  for (int i = 0; i < S; ++i) {
    maxE = std::max(maxE, cut[i + 1] - cut[i]);
    maxN = std::max(maxN, r.off[cut[i + 1]] - r.off[cut[i]]);
    maxC = std::max(maxC, n_chunks_of(cut[i + 1] - cut[i], r.off + cut[i]));
  }
  const int grid = layer_grid_max(h->tuning, std::max(1, maxE * kLayers));
  const auto need = sizes_2d(maxE, maxN, maxC, grid, true);
  DeviceArena* slot_arena[kPipeSlots];
  slot_arena[0] = &h->arena;
  for (int k = 1; k < kPipeSlots; ++k) slot_arena[k] = &h->arena_pipe[k - 1];
  if ((rc = h->arena.reserve(need, h->budget))) return rc;
  for (int k = 1; k < kPipeSlots; ++k) {
    size_t used = h->arena3d.total() + h->arena_bridge.total();
    for (int j = 0; j < kPipeSlots; ++j)
      if (j != k) used += slot_arena[j]->total();
    if ((rc = slot_arena[k]->reserve(need, h->budget > used ? h->budget - used : 0))) return rc;
  }
  // pinned staging: per sub-batch its rebased offsets and chunk table
  std::vector<size_t> st_off(S + 1, 0);
  for (int i = 0; i < S; ++i) {
    const int64_t nci = n_chunks_of(cut[i + 1] - cut[i], r.off + cut[i]);
    st_off[i + 1] = st_off[i] + (((12 * (size_t)(cut[i + 1] - cut[i] + 1) + 4 * (size_t)nci) + 7) & ~size_t(7));
  }
  if ((rc = h->stage.reserve(st_off[S]))) return rc;
  if ((rc = h->flags_host.reserve(4 * kFlagCount * (size_t)S))) return rc;
  cudaError_t e;
  for (auto* st : {&h->copy_in, &h->copy_out}) {
    if (!*st && (e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking)) != cudaSuccess) {
      *st = nullptr;
      return cuda_error(e, "cudaStreamCreate");
    }
  }
  for (auto& ev : h->pipe_events) {
    if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
      ev = nullptr;
      return cuda_error(e, "cudaEventCreate");
    }
  }
  cudaEvent_t* h2d = h->pipe_events;
  cudaEvent_t* comp = h->pipe_events + kPipeSlots;
  cudaEvent_t* d2h = h->pipe_events + 2 * kPipeSlots;
  // the in-copy stream must not overtake work queued earlier on the handle's stream
  for (int k = 0; k < kPipeSlots; ++k)
    if ((e = cudaEventRecord(comp[k], h->stream)) != cudaSuccess ||
        (e = cudaEventRecord(d2h[k], h->stream)) != cudaSuccess)
      return cuda_error(e, "cudaEventRecord");
  int32_t* fh = static_cast<int32_t*>(h->flags_host.p);
  int64_t kernels = 0;
  for (int i = 0; i < S; ++i) {
    const int k = i % kPipeSlots;
    const int32_t e0 = cut[i], Es = cut[i + 1] - e0;
    const int64_t p0 = r.off[e0], Ns = r.off[cut[i + 1]] - p0;
    // staging: rebased offsets, then the chunk table
    int64_t* so = reinterpret_cast<int64_t*>(static_cast<char*>(h->stage.p) + st_off[i]);
    int32_t* sc = reinterpret_cast<int32_t*>(so + (Es + 1));
    sc[0] = 0;
    int32_t* sce = sc + (Es + 1);  // event of each chunk
    for (int32_t j = 0; j <= Es; ++j) so[j] = r.off[e0 + j] - p0;
    for (int32_t j = 0; j < Es; ++j) {
      sc[j + 1] = sc[j] + (int32_t)((so[j + 1] - so[j] + kChunk - 1) / kChunk);
      for (int32_t c = sc[j]; c < sc[j + 1]; ++c) sce[c] = j;
    }
    Run2D sub = r;
    sub.E = Es;
    sub.N = Ns;
    sub.off = so;
    Batch2D b;
    fill_batch_views(h, sub, sc[Es], true, b, slot_arena[k]);
    const size_t n4 = 4 * (size_t)Ns;
    // kernels of both slots stay on the handle's stream: letting the next
    // sub-batch's persistent kernel start beside the draining one measured slower
    cudaStream_t ci = h->copy_in, co = h->copy_out, cs = h->stream;
    if ((e = cudaStreamWaitEvent(ci, comp[k], 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.offsets, so, 8 * (size_t)(Es + 1), cudaMemcpyHostToDevice, ci)) != cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.chunk_start, sc, 4 * (size_t)(Es + 1), cudaMemcpyHostToDevice, ci)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.chunk_ev, sce, 4 * (size_t)sc[Es], cudaMemcpyHostToDevice, ci)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.x, r.x + p0, n4, cudaMemcpyHostToDevice, ci)) != cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.y, r.y + p0, n4, cudaMemcpyHostToDevice, ci)) != cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.layer, r.layer + p0, n4, cudaMemcpyHostToDevice, ci)) != cudaSuccess ||
        (e = cudaMemcpyAsync((void*)b.w, r.w + p0, n4, cudaMemcpyHostToDevice, ci)) != cudaSuccess ||
        (e = cudaEventRecord(h2d[k], ci)) != cudaSuccess)
      return cuda_error(e, "H2D sub-batch");
    if ((e = cudaStreamWaitEvent(cs, h2d[k], 0)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(cs, d2h[k], 0)) != cudaSuccess ||
        (e = cudaMemsetAsync(b.flags + kFlagError, 0, 4, cs)) != cudaSuccess)
      return cuda_error(e, "sub-batch set-up");
    if ((e = launch_clue2d(b, h->p2d, h->tuning, cs, nullptr, &kernels)) != cudaSuccess)
      return cuda_error(e, "launching CLUE kernels");
    if ((e = cudaEventRecord(comp[k], cs)) != cudaSuccess) return cuda_error(e, "cudaEventRecord");
    const clue_outputs* o = r.out;
    if ((e = cudaStreamWaitEvent(co, comp[k], 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o->rho + p0, b.rho, n4, cudaMemcpyDeviceToHost, co)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o->delta + p0, b.delta, n4, cudaMemcpyDeviceToHost, co)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o->nearestHigher + p0, b.nh, n4, cudaMemcpyDeviceToHost, co)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o->isSeed + p0, b.seed, n4, cudaMemcpyDeviceToHost, co)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o->clusterIndex + p0, b.ci, n4, cudaMemcpyDeviceToHost, co)) != cudaSuccess ||
        (e = cudaMemcpyAsync(fh + kFlagCount * (size_t)i, b.flags, 4 * kFlagCount, cudaMemcpyDeviceToHost, co)) !=
            cudaSuccess ||
        (e = cudaEventRecord(d2h[k], co)) != cudaSuccess)
      return cuda_error(e, "D2H sub-batch");
  }
  h->last_run.h2d_bytes = 16 * r.N + 12 * (int64_t)(r.E + S) + 4 * n_chunks_of(r.E, r.off);
  h->last_run.d2h_bytes = 20 * r.N + 4 * kFlagCount * (int64_t)S;
  h->last_run.kernel_launches = kernels;
  // the handle's stream orders after the last copy-out, so later work and
  // clue_synchronize see a finished batch
  for (int k = 0; k < kPipeSlots; ++k)
    if ((e = cudaStreamWaitEvent(h->stream, d2h[k], 0)) != cudaSuccess) return cuda_error(e, "pipelined batch");
  if ((e = cudaStreamSynchronize(h->copy_out)) != cudaSuccess || (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
    return cuda_error(e, "pipelined batch");
  int err = 0;
  for (int i = 0; i < S; ++i) {
    err |= fh[kFlagCount * (size_t)i + kFlagError];
    fh[kFlagCount * (size_t)i + kFlagError] = 0;
  }
  if (err) return set_error(CLUE_EINVAL, "a point has a layer outside [0, %d)", kLayers);
  return CLUE_OK;
}

int run_2d(Handle* h, const Run2D& r) {
  if (r.N == 0) return CLUE_OK;
  if (!r.x || !r.y || !r.layer || !r.w || !r.out || !r.out->rho || !r.out->delta || !r.out->nearestHigher ||
      !r.out->isSeed || !r.out->clusterIndex)
    return set_error(CLUE_EINVAL, "NULL input or output pointer");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  if (r.flags & CLUE_PLAIN) return run_2d_plain(h, r);
  if (!(r.flags & (CLUE_DEVICE_MEMORY | CLUE_NO_PIPELINE | kAsyncHostIO)) && r.N >= 2 * kPipePoints && r.E >= 2)
    return run_2d_pipelined(h, r);
  return run_2d_batched(h, r);
}

}  // namespace

int Handle::profile_batch(int32_t E, const int64_t* off, const float* x, const float* y, const int32_t* layer,
                          const float* w, const clue_outputs* out, float* stage_ms) {
  int rc = validate_offsets(E, off);
  if (rc) return rc;
  if (E == 0 || off[E] == 0) {
    for (int i = 0; i < kStages2D; ++i) stage_ms[i] = 0.f;
    return CLUE_OK;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  cudaEvent_t ev[kStages2D + 1];
  for (int i = 0; i <= kStages2D; ++i) cudaEventCreate(&ev[i]);
  Run2D r{E, off[E], off, x, y, layer, w, out, CLUE_DEVICE_MEMORY | CLUE_NO_GRAPH};
  rc = run_2d_batched(this, r, ev);
  if (rc == CLUE_OK) {
    e = cudaEventSynchronize(ev[kStages2D]);
    if (e != cudaSuccess) rc = cuda_error(e, "profile");
  }
  if (rc == CLUE_OK) {
    for (int i = 0; i < kStages2D; ++i) cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]);
    rc = wait_previous();
    if (rc == CLUE_OK) rc = check_device_flags();
  }
  for (int i = 0; i <= kStages2D; ++i) cudaEventDestroy(ev[i]);
  return rc;
}

int Handle::run_batch(int32_t E, const int64_t* off, const float* x, const float* y, const int32_t* layer,
                      const float* w, const clue_outputs* out, int flags) {
  int rc = validate_offsets(E, off);
  if (rc) return rc;
  if (E == 0) return CLUE_OK;
  Run2D r{E, off[E], off, x, y, layer, w, out, flags};
  return run_2d(this, r);
}

}  // namespace clue

using clue::Handle;
using clue::set_error;
using clue::cuda_error;

extern "C" {

const char* clue_last_error(void) { return clue::g_last_error.c_str(); }

int clue_create(const clue_params* params, size_t budget, int device, void* stream, clue_handle** out) {
  return clue::guarded([&]() -> int {
    if (!params || !out) return set_error(CLUE_EINVAL, "NULL argument");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return set_error(CLUE_EINVAL, "device %d not present (%d devices)", device, ndev);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    e = clue::prepare_clue2d_kernels(device);
    if (e != cudaSuccess) return cuda_error(e, "preparing kernels");
    Handle* h = new Handle();
    h->device = device;
    h->budget = budget ? budget : (size_t(16) << 30);
    h->p2d = clue::make_params2d(params->dc, params->rhoc, params->outlierDeltaFactor);
    if (stream) {
      h->stream = static_cast<cudaStream_t>(stream);
    } else {
      e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        delete h;
        return cuda_error(e, "cudaStreamCreate");
      }
      h->owned_stream = h->stream;
    }
    e = cudaEventCreateWithFlags(&h->done_event, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      delete h;
      return cuda_error(e, "cudaEventCreate");
    }
    *out = reinterpret_cast<clue_handle*>(h);
    return CLUE_OK;
  });
}

int clue_destroy(clue_handle* hh) {
  if (!hh) return CLUE_OK;
  Handle* h = reinterpret_cast<Handle*>(hh);
  cudaSetDevice(h->device);
  if (h->pending) cudaEventSynchronize(h->done_event);
  delete h;
  return CLUE_OK;
}

int clue_set_stream(clue_handle* hh, void* stream) {
  return clue::guarded([&]() -> int {
    if (!hh) return set_error(CLUE_EINVAL, "NULL handle");
    Handle* h = reinterpret_cast<Handle*>(hh);
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    int rc = h->wait_previous();
    if (rc) return rc;
    if (stream) {
      h->stream = static_cast<cudaStream_t>(stream);
      return CLUE_OK;
    }
    if (!h->owned_stream) {
      e = cudaStreamCreateWithFlags(&h->owned_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        h->owned_stream = nullptr;
        return cuda_error(e, "cudaStreamCreate");
      }
    }
    h->stream = h->owned_stream;
    return CLUE_OK;
  });
}

int clue_set_params(clue_handle* hh, const clue_params* p) {
  if (!hh || !p) return set_error(CLUE_EINVAL, "NULL argument");
  Handle* h = reinterpret_cast<Handle*>(hh);
  h->p2d = clue::make_params2d(p->dc, p->rhoc, p->outlierDeltaFactor);
  return CLUE_OK;
}

int clue_run_event(clue_handle* hh, int32_t n, const float* x, const float* y, const int32_t* layer,
                   const float* weight, const clue_outputs* out, int flags) {
  return clue::guarded([&]() -> int {
    if (!hh) return set_error(CLUE_EINVAL, "NULL handle");
    if (n < 0) return set_error(CLUE_EINVAL, "n < 0");
    int64_t off[2] = {0, n};
    return reinterpret_cast<Handle*>(hh)->run_batch(1, off, x, y, layer, weight, out, flags & ~CLUE_PLAIN);
  });
}

int clue_run_batch(clue_handle* hh, int32_t n_events, const int64_t* event_offsets, const float* x, const float* y,
                   const int32_t* layer, const float* weight, const clue_outputs* out, int flags) {
  return clue::guarded([&]() -> int {
    if (!hh) return set_error(CLUE_EINVAL, "NULL handle");
    return reinterpret_cast<Handle*>(hh)->run_batch(n_events, event_offsets, x, y, layer, weight, out, flags);
  });
}

int clue_last_run_stats(clue_handle* hh, clue_run_stats* stats) {
  if (!hh || !stats) return set_error(CLUE_EINVAL, "NULL argument");
  *stats = reinterpret_cast<const Handle*>(hh)->last_run;
  return CLUE_OK;
}

int clue_synchronize(clue_handle* hh) {
  return clue::guarded([&]() -> int {
    if (!hh) return set_error(CLUE_EINVAL, "NULL handle");
    Handle* h = reinterpret_cast<Handle*>(hh);
    cudaSetDevice(h->device);
    int rc = h->wait_previous();
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
    return h->check_device_flags();
  });
}

size_t clue_required_bytes(int32_t n_events, int64_t n_points, int flags) {
  if (n_events < 0 || n_points < 0) return 0;
  int64_t nchunks = n_points / clue::kChunk + n_events;
  return clue::required_bytes_2d(n_events, n_points, nchunks, 1216, !(flags & CLUE_DEVICE_MEMORY));
}

int clue_profile_batch(clue_handle* hh, int32_t n_events, const int64_t* event_offsets, const float* x,
                       const float* y, const int32_t* layer, const float* weight, const clue_outputs* out,
                       float* stage_ms) {
  return clue::guarded([&]() -> int {
    if (!hh || !out || !stage_ms) return set_error(CLUE_EINVAL, "NULL argument");
    return reinterpret_cast<Handle*>(hh)->profile_batch(n_events, event_offsets, x, y, layer, weight, out, stage_ms);
  });
}

int clue_get_tuning(clue_handle* hh, clue_tuning* t) {
  if (!hh || !t) return set_error(CLUE_EINVAL, "NULL argument");
  Handle* h = reinterpret_cast<Handle*>(hh);
  t->threads = h->tuning.threads;
  t->layer_capacity = h->tuning.layer_capacity;
  t->work_tile_cm = h->tuning.work_tile_cm;
  t->ctas_per_sm = h->tuning.ctas_per_sm;
  t->big_threads = h->tuning.big_threads;
  t->big_capacity = h->tuning.big_capacity;
  return CLUE_OK;
}

int clue_set_tuning(clue_handle* hh, const clue_tuning* t) {
  if (!hh || !t) return set_error(CLUE_EINVAL, "NULL argument");
  if (t->threads != 128 && t->threads != 256 && t->threads != 512 && t->threads != 1024)
    return set_error(CLUE_EINVAL, "threads must be 128, 256, 512 or 1024");
  if (t->layer_capacity < 32 || clue::layer_smem_bytes(clue::Tuning2D{t->threads, t->layer_capacity}) > 227 * 1024 - 1024)
    return set_error(CLUE_EINVAL, "layer_capacity %d does not fit in shared memory", t->layer_capacity);
  if (t->work_tile_cm != 0.f) return set_error(CLUE_EINVAL, "work_tile_cm is reserved and must be 0");
  if (t->ctas_per_sm < 0 || t->ctas_per_sm > 8) return set_error(CLUE_EINVAL, "ctas_per_sm must be in [0, 8]");
  if (t->big_threads != 0 && t->big_threads != 128 && t->big_threads != 256 && t->big_threads != 512 &&
      t->big_threads != 1024)
    return set_error(CLUE_EINVAL, "big_threads must be 0, 128, 256, 512 or 1024");
  if (t->big_threads != 0 &&
      clue::layer_smem_bytes(clue::Tuning2D{t->big_threads, t->big_capacity}) > 227 * 1024 - 1024)
    return set_error(CLUE_EINVAL, "big_capacity %d does not fit in shared memory", t->big_capacity);
  Handle* h = reinterpret_cast<Handle*>(hh);
  h->tuning.threads = t->threads;
  h->tuning.layer_capacity = t->layer_capacity;
  h->tuning.work_tile_cm = t->work_tile_cm;
  h->tuning.ctas_per_sm = t->ctas_per_sm;
  h->tuning.big_threads = t->big_threads;
  h->tuning.big_capacity = t->big_capacity;
  return CLUE_OK;
}

}  // extern "C"
