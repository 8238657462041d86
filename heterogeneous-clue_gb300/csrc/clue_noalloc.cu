// clue_run_event_noalloc: CLUE 2D on one event without allocating anything.
//
// Some callers cannot call cudaMalloc: host frameworks that hand their whole
// device-memory budget to their own pool allocator up front, real-time or
// embedded callers that must not touch the allocator after start-up, and
// code paths that run while another component owns the device's memory
// management.  For them this entry point takes device pointers for inputs and
// outputs and does all of its work in one fixed scratch area that is part of
// the library image: a file-scope __device__ array.
//
// Limits and rules (also in include/clue.h):
//  * at most kNoAllocMaxPoints points per call; larger events get CLUE_EINVAL;
//  * the runtime loads a library's device code, and creates its __device__
//    arrays, lazily: on a device, the first use of this file's code creates
//    the 14 MB array, and the first launch of each kernel loads its code.
//    Make the first call on each device at start-up, before the caller's
//    framework reserves the device's memory for its pool; a call with n == 0
//    does exactly that set-up (array, kernel code, shared-memory opt-in)
//    and nothing else.  Make it outside any stream capture.  The array then
//    stays until the process exits;
//  * every call looks the array's device address up again (cheap once the
//    code is loaded), so a reset of the device's context in between does not
//    leave a stale address behind;
//  * every call on a device uses the same array: calls that overlap on the
//    GPU (other streams or threads) race and corrupt each other; the call
//    synchronises its stream before it returns;
//  * the array keeps whatever the previous call left; everything the
//    pipeline needs at zero is cleared at the start of each call.
// No cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/clue.h"
#include "clue_internal.h"
#include "clue_runtime.h"

namespace clue {
namespace {

constexpr int64_t kNoAllocMaxPoints = 1 << 18;  // 262,144 points per event
// Per-CTA HBM tile tables of the spill path: launch_clue2d never launches more
// layer-kernel CTAs than (event, layer) items, i.e. 100 for one event.
constexpr int kNoAllocMaxGrid = kLayers;
constexpr int64_t kNoAllocMaxChunks = kNoAllocMaxPoints / kChunk + 1;

// Byte layout of the scratch area (every piece 256-byte aligned).
constexpr size_t al(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kOffOffsets = 0;                                              // int64[2]
constexpr size_t kOffChunkStart = kOffOffsets + al(16);                        // int32[2]
constexpr size_t kOffLcnt = kOffChunkStart + al(8);                            // int32[100]
constexpr size_t kOffLstart = kOffLcnt + al(4 * kLayers);                      // int32[100]
constexpr size_t kOffCursor = kOffLstart + al(4 * kLayers);                    // int32[100]
constexpr size_t kOffOrder = kOffCursor + al(4 * kLayers);                     // int32[100 + 2 * size classes]
constexpr size_t kOffFlags = kOffOrder + al(4 * (kLayers + 2 * kSizeBuckets));  // int32[kFlagCount]
constexpr size_t kOffChunkSeeds = kOffFlags + al(4 * kFlagCount);              // int32[chunks]
constexpr size_t kOffChunkBase = kOffChunkSeeds + al(4 * kNoAllocMaxChunks);   // int32[chunks]
constexpr size_t kOffGx = kOffChunkBase + al(4 * kNoAllocMaxChunks);           // 4 x [N] grouped copies
constexpr size_t kOffSpRec = kOffGx + 4 * al(4 * kNoAllocMaxPoints);           // 16 B x N spill records
constexpr size_t kOffSpNh = kOffSpRec + al(16 * kNoAllocMaxPoints);            // int32[N]
constexpr size_t kOffSpQord = kOffSpNh + al(4 * kNoAllocMaxPoints);            // int32[N]
constexpr size_t kOffSpTbl = kOffSpQord + al(4 * kNoAllocMaxPoints);           // per-CTA HBM tile tables
constexpr size_t kNoAllocBytes = kOffSpTbl + al(4 * (size_t)kTableStride * kNoAllocMaxGrid);

// The scratch area itself.  In host code this name is only a stand-in for
// the symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

__global__ void k_noalloc_event_header(int64_t* offsets, int32_t* chunk_start, int64_t n) {
  offsets[0] = 0;
  offsets[1] = n;
  chunk_start[0] = 0;
  chunk_start[1] = (int32_t)((n + kChunk - 1) / kChunk);
}

// Set-up on the current device: the scratch area's device address (looked
// up on every call: cheap once the code is loaded, and never stale after a
// context reset) and the kernels' code and shared-memory opt-in.
int noalloc_scratch(unsigned char** out) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scratch)");
  cudaFuncAttributes a;
  e = cudaFuncGetAttributes(&a, k_noalloc_event_header);
  if (e != cudaSuccess) return cuda_error(e, "loading kernels");
  e = prepare_clue2d_kernels(device);
  if (e != cudaSuccess) return cuda_error(e, "preparing kernels");
  *out = static_cast<unsigned char*>(p);
  return CLUE_OK;
}

}  // namespace
}  // namespace clue

using namespace clue;

extern "C" int clue_run_event_noalloc(const clue_params* params, int32_t n, const float* x, const float* y,
                                      const int32_t* layer, const float* weight, const clue_outputs* out,
                                      void* cuda_stream) {
  if (n < 0) return set_error(CLUE_EINVAL, "n < 0");
  if (n > kNoAllocMaxPoints)
    return set_error(CLUE_EINVAL, "clue_run_event_noalloc: %d points exceed its fixed scratch (at most %lld)", n,
                     (long long)kNoAllocMaxPoints);
  if (n > 0) {
    if (!params || !out || !out->rho || !out->delta || !out->nearestHigher || !out->isSeed || !out->clusterIndex)
      return set_error(CLUE_EINVAL, "NULL argument");
    if (!x || !y || !layer || !weight) return set_error(CLUE_EINVAL, "NULL input array");
  }
  unsigned char* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  if (n == 0) return CLUE_OK;  // the warm-up call: set-up only, every pointer may be NULL
  cudaError_t e;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

  Batch2D b;
  b.n_events = 1;
  b.n_points = n;
  b.n_chunks = (int32_t)((n + kChunk - 1) / kChunk);
  b.offsets = reinterpret_cast<const int64_t*>(base + kOffOffsets);
  b.chunk_start = reinterpret_cast<const int32_t*>(base + kOffChunkStart);
  b.x = x;
  b.y = y;
  b.layer = layer;
  b.w = weight;
  b.rho = out->rho;
  b.delta = out->delta;
  b.nh = out->nearestHigher;
  b.seed = out->isSeed;
  b.ci = out->clusterIndex;
  b.lcnt = reinterpret_cast<int32_t*>(base + kOffLcnt);
  b.lstart = reinterpret_cast<int32_t*>(base + kOffLstart);
  b.cursor = reinterpret_cast<int32_t*>(base + kOffCursor);
  b.flags = reinterpret_cast<int32_t*>(base + kOffFlags);
  b.order = reinterpret_cast<int32_t*>(base + kOffOrder);
  b.size_hist = b.order + kLayers;
  b.chunk_seeds = reinterpret_cast<int32_t*>(base + kOffChunkSeeds);
  b.chunk_base = reinterpret_cast<int32_t*>(base + kOffChunkBase);
  const size_t plane = al(4 * kNoAllocMaxPoints);
  b.gx = reinterpret_cast<float*>(base + kOffGx);
  b.gy = reinterpret_cast<float*>(base + kOffGx + plane);
  b.gw = reinterpret_cast<float*>(base + kOffGx + 2 * plane);
  b.gid = reinterpret_cast<int32_t*>(base + kOffGx + 3 * plane);
  b.sp[0] = reinterpret_cast<float*>(base + kOffSpRec);
  b.sp[4] = reinterpret_cast<float*>(base + kOffSpNh);
  b.sp[5] = reinterpret_cast<float*>(base + kOffSpQord);
  b.sp_tbl = reinterpret_cast<int32_t*>(base + kOffSpTbl);  // kNoAllocMaxGrid tables: see its definition

  Tuning2D t;  // the default decomposition
  const Params2D p = make_params2d(params->dc, params->rhoc, params->outlierDeltaFactor);

  k_noalloc_event_header<<<1, 1, 0, s>>>(const_cast<int64_t*>(b.offsets), const_cast<int32_t*>(b.chunk_start), n);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "launching CLUE kernels");
  if ((e = cudaMemsetAsync(b.flags + kFlagError, 0, sizeof(int32_t), s)) != cudaSuccess)
    return cuda_error(e, "clearing status");
  if ((e = launch_clue2d(b, p, t, s)) != cudaSuccess) return cuda_error(e, "launching CLUE kernels");
  int32_t err_word = 0;
  if ((e = cudaMemcpyAsync(&err_word, b.flags + kFlagError, sizeof(int32_t), cudaMemcpyDeviceToHost, s)) !=
      cudaSuccess)
    return cuda_error(e, "reading status");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  if (err_word) return set_error(CLUE_EINVAL, "a point has a layer outside [0, %d)", kLayers);
  return CLUE_OK;
}
