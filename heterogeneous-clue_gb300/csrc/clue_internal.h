// Internal declarations shared by the CUDA kernels and the host runtime.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstddef>
#include <cstdint>

namespace clue {

// NVTX range over a scope: marks where each pipeline stage is queued on the
// host timeline (Nsight Systems / Nsight Compute NVTX filters).  Inside a
// stream capture the ranges mark the capture; a graph replay is one range.
// With no tool attached a range costs a few nanoseconds.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Tile grid of the reference (src/serial/DataFormats/LayerTilesConstants.h:7-26):
// 100 layers, x and y in [-250, 250] cm, 5 cm tiles -> 100 x 100 per layer.
constexpr int kLayers = 100;
constexpr int kGridCols = 100;
constexpr int kTiles = kGridCols * kGridCols;
constexpr int kTableInts = kTiles + 1;
// Bytes of the on-chip 16-bit tile table (a multiple of 16).
constexpr int kSmemTableBytes = ((kTableInts * 2 + 15) / 16) * 16;
// Per-CTA stride of the HBM tile tables (32-bit counts), a multiple of 16 bytes.
constexpr int kTableStride = ((kTableInts * 4 + 15) / 16) * 4;
// Points per event-aligned chunk of the streaming kernels (count, scatter, seed ranks).
constexpr int kChunk = 4096;
constexpr int kChunkThreads = 512;
// Size classes of the largest-first layer order (16 points per class).
constexpr int kSizeBuckets = 256;

// Device-side status words of one run.
enum FlagSlot : int {
  kFlagGrouped = 0,
  kFlagError = 1,
  kFlagTicket = 2,
  kFlagSpilled = 3,
  kFlagTicket2 = 4,   // ticket of the large-layer pass
  kFlagBigCount = 5,  // layers left to the large-layer pass
  kFlagOrdered = 6,   // non-empty layers in the size order
  kFlagCount = 8
};

struct Params2D {
  float dc, rhoc, odf;
  float dm;    // odf * dc, as the reference computes it (float product)
  float t_dc;  // largest float t >= 0 with sqrtf(t) <= dc, or -1 when none
  float t_dm;  // same for dm
  float t_dm_next;  // next float above t_dm (or -1)
};

// Host: fill Params2D from the three reference parameters.
Params2D make_params2d(float dc, float rhoc, float odf);
// Largest float t >= 0 with sqrtf(t) <= d (correctly rounded sqrt), or -1.
float sqrt_le_threshold(float d);

struct Tuning2D {
  int threads = 256;
  int layer_capacity = 1536;
  float work_tile_cm = 0.f;
  int ctas_per_sm = 0;
  int big_threads = 512;     // second pass for layers above layer_capacity (0 = none)
  int big_capacity = 4096;
};

// Device views of one 2D batch.  All [N] arrays are in the caller's point order
// (inputs/outputs) or in grouped-by-(event, layer) order (scratch).
struct Batch2D {
  int32_t n_events = 0;
  int64_t n_points = 0;
  int32_t n_chunks = 0;
  const int64_t* offsets = nullptr;      // [E+1]
  const int32_t* chunk_start = nullptr;  // [E+1] first chunk of each event
  const int32_t* chunk_ev = nullptr;     // [n_chunks] event of each chunk (nullptr: searched in chunk_start)
  const float* x = nullptr;
  const float* y = nullptr;
  const int32_t* layer = nullptr;
  const float* w = nullptr;
  float* rho = nullptr;
  float* delta = nullptr;
  int32_t* nh = nullptr;
  int32_t* seed = nullptr;
  int32_t* ci = nullptr;
  // scratch
  int32_t* lcnt = nullptr;    // [E*100] points per (event, layer)
  int32_t* lstart = nullptr;  // [E*100] first grouped position of (event, layer)
  int32_t* cursor = nullptr;  // [E*100]
  int32_t use_order = 0;         // set per launch: take the layers in `order`
  int32_t* order = nullptr;      // [E*100] non-empty (event, layer) items, largest first
  int32_t* size_hist = nullptr;  // [2*kSizeBuckets] layers per size class, then cursors
  float* gx = nullptr;        // [N] grouped copies, event-local index in gid
  float* gy = nullptr;
  float* gw = nullptr;
  int32_t* gid = nullptr;
  float* sp[8] = {};          // [N] each: HBM home of layers larger than layer_capacity
  int32_t* sp_tbl = nullptr;  // [grid * kTableInts]
  int32_t* chunk_seeds = nullptr;  // [n_chunks]
  int32_t* chunk_base = nullptr;   // [n_chunks]
  int32_t* flags = nullptr;        // [kFlagCount]
};

// Grid of the layer kernel for a tuning (needs the current device).
int layer_grid(const Tuning2D& t, int n_items);
// The larger grid of the two layer passes (sizes the per-CTA HBM tables).
int layer_grid_max(const Tuning2D& t, int n_items);
size_t layer_smem_bytes(const Tuning2D& t);

// Opts the layer kernels into the device's full shared memory and loads the
// code of every kernel of the 2D pipeline on the current device (outside any
// stream capture; again after the device's context was reset).
cudaError_t prepare_clue2d_kernels(int device);

constexpr int kStages2D = 7;
// Queues the whole 2D pipeline of one batch on `s`.  With `stage_events`
// (kStages2D + 1 events) an event is recorded before each stage and after the
// last; `kernels`, when given, is increased by the number of kernels queued.
cudaError_t launch_clue2d(const Batch2D& b, const Params2D& p, const Tuning2D& t, cudaStream_t s,
                          cudaEvent_t* stage_events = nullptr, int64_t* kernels = nullptr);

// Adds an order-sensitive digest of n_words 32-bit words to *d_out.
cudaError_t launch_digest(const void* words, int64_t n_words, unsigned long long* d_out, cudaStream_t s);

// ---------------------------------------------------------------- CLUE3D --
struct Params3D {
  int n_layers;
  int dens_sib, nh_sib;
  int dens_same, nh_same;
  float dens_thr;         // density_xy_distance_sqr
  float kdf;              // kernel_density_factor
  float crit_xy, crit_z, crit_rho, crit_self, outlier_mult;
  float out_thr;          // outlier_mult * crit_xy (float product)
  // binning constants, computed on the host exactly as the reference does
  float eta_r;            // nEtaBins / (maxEta - minEta)
  float phi_r;            // (float)(nPhiBins * M_1_PI * 0.5f)
  float o2pi;             // (float)(1 / (2 pi))
  float pi_f;             // (float)M_PI
  float twopi_f;          // (float)(2 pi)
};

struct Batch3D {
  int32_t n_events = 0;
  int64_t n_points = 0;
  int32_t n_rows = 0;  // rows (layer, eta) per event: n_layers * 34 + 1
  const int64_t* offsets = nullptr;  // [E+1]
  const int32_t* blk_ev = nullptr;   // [ceil(N / 256)] event of each 256-cluster block's first cluster
  const float* z = nullptr;
  const float* eta = nullptr;
  const float* phi = nullptr;
  const float* roa = nullptr;
  const float* radius = nullptr;
  const int32_t* layer = nullptr;
  const float* energy = nullptr;
  const int32_t* sil = nullptr;
  float* rho = nullptr;
  float* delta_t = nullptr;
  int32_t* delta_l = nullptr;
  int32_t* nh_l = nullptr;
  int32_t* nh_i = nullptr;
  int32_t* seed = nullptr;
  int32_t* ti = nullptr;
  // scratch
  int32_t* key = nullptr;      // [N] flat (layer, eta, phi) bin
  int32_t* row_cnt = nullptr;  // [E * n_rows + 1]
  int32_t* row_start = nullptr;// [E * n_rows + 1]
  int32_t* arr = nullptr;      // [N] arrival slot of each cluster in its row
  int32_t* sorted = nullptr;   // [N] event-local index, by (row, phi bin, index)
  int32_t* scol = nullptr;     // [N] phi bin of sorted entries
  float4* cand = nullptr;      // [N] by sorted position: {roa, phi, energy, rho} of the entry
  float4* qrec = nullptr;      // [N] by sorted position: {z, roa * z, density threshold, layer | etaBin << 11 | phiBin << 17}
  float4* tcand = nullptr;     // [N] cand records by scatter position
  float4* tqrec = nullptr;     // [N] qrec records by scatter position
  int32_t* tmp = nullptr;      // [N]
  int32_t* par = nullptr;      // [N]
  int32_t* ev_seeds = nullptr; // [E] tracksters per event
  unsigned long long* row_mask = nullptr;  // [E * n_rows * 2] phi columns present in each row; bit 127: a column repeats
  unsigned long long* row_rep = nullptr;   // [E * n_rows * 2] columns holding a second entry; bit 127: a third
  int32_t* flags = nullptr;    // [kFlagCount]
};

cudaError_t launch_clue3d(const Batch3D& b, const Params3D& p, cudaStream_t s);

}  // namespace clue
