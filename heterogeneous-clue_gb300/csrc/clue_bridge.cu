// 2D -> 3D bridge: the layer clusters of a clustered 2D batch, built on the
// device as CLUE3D input (a ClusterCollection per event,
// src/serial/DataFormats/ClusterCollection.h:6-19).  The reference has no such
// step (its CLUE3D reads raw3D files, src/serial/bin/Source.cc:43-60), so the
// definition is this file's:
//
//   * layer cluster c of event e = the 2D points with clusterIndex == c; the
//     clusters of an event keep the 2D ids' order (seed rank in index order);
//   * energy = sum of the weights, position = weight-weighted mean of x, y.
//     The sums are exact fixed-point integers (weights in units of 2^-24,
//     weight * coordinate in units of 2^-16, both rounded to nearest), so
//     they do not depend on the order of accumulation and the GPU result is
//     deterministic; the division and conversions are IEEE double;
//   * layer = the seed's layer, z = layer_z[layer], r = |(x, y)|,
//     r_over_absz = r / |z|, eta = asinh(z / max(r, 1e-9)), phi = atan2(y, x),
//     radius and isSilicon constant.  Clusters with zero total weight take the
//     seed's position.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "clue_runtime.h"

namespace clue {
namespace {

constexpr double kWScale = 16777216.0;  // 2^24
constexpr double kPScale = 65536.0;     // 2^16

enum BridgeSlot { B_OFF, B_COFF, B_COUNT, B_ACC, B_SEED, B_LZ, B_FLAGS, B_CEV, B_SLOTS };

// Points per block of the point kernels: each block finds the event of its
// first point once and then follows event boundaries forwards.
constexpr int kBridgeChunk = 4096;
constexpr int kBridgeThreads = 256;

int chunks_for(int64_t n) { return (int)((n + kBridgeChunk - 1) / kBridgeChunk); }

// Round-to-nearest-even of m * 2^sh for m < 2^48 and sh <= 14 (fits 63 bits).
__device__ __forceinline__ unsigned long long round_shift(unsigned long long m, int sh) {
  if (sh >= 0) return m << sh;
  if (-sh > 49) return 0;  // below one half
  const int sr = -sh;
  const unsigned long long q = m >> sr, rem = m & ((1ull << sr) - 1), half = 1ull << (sr - 1);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

// Fixed-point weight, round(w * 2^24) as the double formula gives it: on the
// integer significand (the product w * 2^24 is exact), without FP64 or a
// float-to-int64 conversion; NaN, infinities and huge weights take the
// double formula.
__device__ __forceinline__ unsigned long long fx_weight(float w) {
  const unsigned uw = __float_as_uint(w);
  int ew = (uw >> 23) & 0xff;
  unsigned long long mw = uw & 0x7fffffu;
  const int sh = (ew ? ew : 1) - 150 + 24;  // value = mw * 2^sh
  if (ew == 0xff || sh > 30) return (unsigned long long)__double2ll_rn((double)w * kWScale);
  if (ew) mw |= 0x800000u;
  const unsigned long long q = round_shift(mw, sh);
  return (uw >> 31) ? (0ull - q) : q;
}

// Fixed-point weighted coordinate, round(w * v * 2^16) to nearest even, as
// the double formula gives it (the double product of two floats is exact):
// computed on the integer significands (a 48-bit product, shifted with
// round-half-even), without FP64, which is slow on this GPU.  Infinities,
// NaN and products that may not fit 63 bits take the double formula.
__device__ __forceinline__ unsigned long long fx_pos(float w, float v) {
  const unsigned uw = __float_as_uint(w), uv = __float_as_uint(v);
  int ew = (uw >> 23) & 0xff, ev = (uv >> 23) & 0xff;
  unsigned long long mw = uw & 0x7fffffu, mv = uv & 0x7fffffu;
  if (ew == 0xff || ev == 0xff) return (unsigned long long)__double2ll_rn((double)w * (double)v * kPScale);
  if (ew) mw |= 0x800000u; else ew = 1;
  if (ev) mv |= 0x800000u; else ev = 1;
  const unsigned long long m = mw * mv;          // below 2^48
  const int sh = (ew - 150) + (ev - 150) + 16;   // value = m * 2^sh
  if (sh > 14) return (unsigned long long)__double2ll_rn((double)w * (double)v * kPScale);
  const unsigned long long q = round_shift(m, sh);
  return ((uw ^ uv) >> 31) ? (0ull - q) : q;
}

// Points of a thread per round (loads of a round are issued together).
constexpr int kBridgePer = 8;
constexpr int kBridgeRounds = kBridgeChunk / (kBridgeThreads * kBridgePer);
static_assert(kBridgeRounds * kBridgeThreads * kBridgePer == kBridgeChunk, "chunk layout");

// Seeds per event: each block counts its chunk's seeds per event in shared
// memory (a chunk touches few events) and adds each count once; seeds of
// events beyond the first kBlockEvents of the chunk go to global memory.
constexpr int kBlockEvents = 32;

__global__ void __launch_bounds__(kBridgeThreads) k_bridge_count(int64_t N, const int64_t* __restrict__ off,
                                                                   const int32_t* __restrict__ chunk_ev,
                                                                   const int32_t* __restrict__ seed,
                                                                   int32_t* __restrict__ counts) {
  __shared__ int32_t s_cnt[kBlockEvents];
  if (threadIdx.x < kBlockEvents) s_cnt[threadIdx.x] = 0;
  const int64_t c0 = (int64_t)blockIdx.x * kBridgeChunk;
  const int32_t e0 = chunk_ev[blockIdx.x];
  int32_t e = e0;
  int64_t next = off[e + 1];  // first point after event e
  __syncthreads();
  for (int rd = 0; rd < kBridgeRounds; ++rd) {
    const int64_t i0 = c0 + (int64_t)rd * kBridgeThreads * kBridgePer + threadIdx.x;
    int32_t sv[kBridgePer];
#pragma unroll
    for (int j = 0; j < kBridgePer; ++j) {
      const int64_t i = i0 + (int64_t)j * kBridgeThreads;
      sv[j] = i < N ? seed[i] : 0;
    }
#pragma unroll
    for (int j = 0; j < kBridgePer; ++j) {
      const int64_t i = i0 + (int64_t)j * kBridgeThreads;
      if (i < N && sv[j]) {
        while (next <= i) next = off[++e + 1];  // i grows with (rd, j)
        if (e - e0 < kBlockEvents) atomicAdd(&s_cnt[e - e0], 1);
        else atomicAdd(&counts[e], 1);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < kBlockEvents && s_cnt[threadIdx.x]) atomicAdd(&counts[e0 + threadIdx.x], s_cnt[threadIdx.x]);
}

// The sums of a cluster are exact integers, so they may be added in any
// grouping: each thread takes kRun consecutive points (read 4 at a time with
// 16-byte loads), keeps running sums while the cluster stays the same (a
// cluster's points are mostly consecutive), and makes the three atomic
// additions once per run.
constexpr int kRun = kBridgeChunk / kBridgeThreads;  // 16 points per thread
static_assert(kRun % 4 == 0, "vector loads");

__global__ void __launch_bounds__(kBridgeThreads) k_bridge_accumulate(
    int64_t N, const int64_t* __restrict__ off, const int32_t* __restrict__ chunk_ev,
    const int64_t* __restrict__ coff, const float* __restrict__ x, const float* __restrict__ y,
    const float* __restrict__ w, const int32_t* __restrict__ seed, const int32_t* __restrict__ ci,
    unsigned long long* __restrict__ acc, int32_t* __restrict__ seed_of, int32_t* __restrict__ flags) {
  const int64_t i0 = (int64_t)blockIdx.x * kBridgeChunk + (int64_t)threadIdx.x * kRun;
  if (i0 >= N) return;
  int32_t e = chunk_ev[blockIdx.x];
  int64_t next = off[e + 1];  // first point after event e
  while (next <= i0) next = off[++e + 1];
  int64_t cbase = coff[e], ccount = coff[e + 1] - cbase;
  int32_t cur = -1;
  unsigned long long s0 = 0, s1 = 0, s2 = 0;
  auto flush = [&]() {
    if (cur >= 0) {
      atomicAdd(&acc[3 * (int64_t)cur], s0);
      atomicAdd(&acc[3 * (int64_t)cur + 1], s1);
      atomicAdd(&acc[3 * (int64_t)cur + 2], s2);
    }
  };
  // 16-byte loads when the run is whole and every array is 16-byte aligned
  // (i0 is a multiple of 16 points); otherwise points are read one by one
  const bool vec = i0 + kRun <= N && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) |
                                      reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(seed) |
                                      reinterpret_cast<uintptr_t>(ci)) & 15) == 0;
  // unrolled, so that the loads of later groups of four are issued before the
  // earlier groups' fixed-point work (1,000 HGCAL events: 5.74 -> 5.48 ms)
#pragma unroll
  for (int k0 = 0; k0 < kRun; k0 += 4) {
    int32_t cv[4], sv[4];
    float wv[4], xv[4], yv[4];
    if (vec) {
      const int4 c4 = *reinterpret_cast<const int4*>(ci + i0 + k0);
      const int4 s4 = *reinterpret_cast<const int4*>(seed + i0 + k0);
      const float4 w4 = *reinterpret_cast<const float4*>(w + i0 + k0);
      const float4 x4 = *reinterpret_cast<const float4*>(x + i0 + k0);
      const float4 y4 = *reinterpret_cast<const float4*>(y + i0 + k0);
      cv[0] = c4.x; cv[1] = c4.y; cv[2] = c4.z; cv[3] = c4.w;
      sv[0] = s4.x; sv[1] = s4.y; sv[2] = s4.z; sv[3] = s4.w;
      wv[0] = w4.x; wv[1] = w4.y; wv[2] = w4.z; wv[3] = w4.w;
      xv[0] = x4.x; xv[1] = x4.y; xv[2] = x4.z; xv[3] = x4.w;
      yv[0] = y4.x; yv[1] = y4.y; yv[2] = y4.z; yv[3] = y4.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i = i0 + k0 + j;
        const bool in = i < N;
        cv[j] = in ? ci[i] : -1;
        sv[j] = in ? seed[i] : 0;
        wv[j] = in ? w[i] : 0.f;
        xv[j] = in ? x[i] : 0.f;
        yv[j] = in ? y[i] : 0.f;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = i0 + k0 + j;
      if (i >= N) break;
      if (next <= i) {
        while (next <= i) next = off[++e + 1];
        cbase = coff[e];
        ccount = coff[e + 1] - cbase;
      }
      int32_t g = -1;
      if (cv[j] >= 0) {
        if (cv[j] >= ccount) atomicExch(&flags[kFlagError], 1);
        else g = (int32_t)(cbase + cv[j]);
      }
      if (g != cur) {
        flush();
        cur = g;
        s0 = s1 = s2 = 0;
      }
      if (g >= 0) {
        s0 += fx_weight(wv[j]);
        s1 += fx_pos(wv[j], xv[j]);
        s2 += fx_pos(wv[j], yv[j]);
        if (sv[j]) seed_of[g] = (int32_t)i;
      }
    }
  }
  flush();
}

__global__ void k_bridge_finalize(int64_t C, const unsigned long long* __restrict__ acc,
                                  const int32_t* __restrict__ seed_of, const float* __restrict__ x,
                                  const float* __restrict__ y, const int32_t* __restrict__ layer,
                                  const float* __restrict__ layer_z, int32_t n_layers, float radius, int32_t sil,
                                  clue_layer_clusters o, int32_t* __restrict__ flags) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < C; g += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = seed_of[g];
    int32_t L = layer[s];
    if (L < 0 || L >= n_layers) {
      atomicExch(&flags[kFlagError], 2);
      L = 0;
    }
    const long long sw = (long long)acc[3 * g];
    float xb, yb;
    if (sw != 0) {
      const double den = (double)sw;
      xb = __double2float_rn((double)(long long)acc[3 * g + 1] * (kWScale / kPScale) / den);
      yb = __double2float_rn((double)(long long)acc[3 * g + 2] * (kWScale / kPScale) / den);
    } else {
      xb = x[s];
      yb = y[s];
    }
    const float z = layer_z[L];
    const double xd = xb, yd = yb;
    const double r = sqrt(xd * xd + yd * yd);
    o.x[g] = xb;
    o.y[g] = yb;
    o.z[g] = z;
    o.r_over_absz[g] = __double2float_rn(r / fabs((double)z));
    o.eta[g] = __double2float_rn(asinh((double)z / fmax(r, 1e-9)));
    o.phi[g] = __double2float_rn(atan2(yd, xd));
    o.radius[g] = radius;
    o.layer[g] = L;
    o.energy[g] = __double2float_rn((double)sw / kWScale);
    o.isSilicon[g] = sil;
  }
}

int check_offsets(int32_t E, const int64_t* off, const char* what) {
  if (E < 0) return set_error(CLUE_EINVAL, "n_events < 0");
  if (E == 0) return CLUE_OK;
  if (!off) return set_error(CLUE_EINVAL, "%s is NULL", what);
  if (off[0] != 0) return set_error(CLUE_EINVAL, "%s[0] must be 0", what);
  for (int32_t e = 0; e < E; ++e)
    if (off[e + 1] < off[e]) return set_error(CLUE_EINVAL, "%s must be non-decreasing", what);
  if (off[E] > INT32_MAX) return set_error(CLUE_EINVAL, "more than 2^31-1 entries in %s", what);
  return CLUE_OK;
}

// Event of the first point of each chunk of kBridgeChunk points (empty
// events own no point; the event of a point is the last e with off[e] <= i).
void chunk_events(int32_t E, const int64_t* off, int nch, int32_t* cev) {
  int32_t e = 0;
  for (int c = 0; c < nch; ++c) {
    const int64_t i = (int64_t)c * kBridgeChunk;
    while (e + 1 < E && off[e + 1] <= i) ++e;
    cev[c] = e;
  }
}

int grid_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
}

size_t bridge_budget(const Handle* h) {
  const size_t used = h->arena.total() + h->arena3d.total();
  return h->budget > used ? h->budget - used : 0;
}

}  // namespace
}  // namespace clue

using clue::Handle;
using clue::cuda_error;
using clue::set_error;

extern "C" {

int clue_bridge_count(clue_handle* hh, int32_t E, const int64_t* off, const int32_t* isSeed,
                      int64_t* cluster_offsets) {
  return clue::guarded([&]() -> int {
    if (!hh || !cluster_offsets) return set_error(CLUE_EINVAL, "NULL argument");
    int rc = clue::check_offsets(E, off, "event_offsets");
    if (rc) return rc;
    cluster_offsets[0] = 0;
    if (E == 0) return CLUE_OK;
    const int64_t N = off[E];
    if (N > 0 && !isSeed) return set_error(CLUE_EINVAL, "isSeed is NULL");
    Handle* h = reinterpret_cast<Handle*>(hh);
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    if ((rc = h->wait_previous())) return rc;
    std::vector<size_t> need(clue::B_SLOTS, 0);
    need[clue::B_OFF] = 8 * (size_t)(E + 1);
    need[clue::B_COUNT] = 4 * (size_t)E;
    const int nch = clue::chunks_for(N);
    need[clue::B_CEV] = 4 * (size_t)std::max(nch, 1);
    if ((rc = h->arena_bridge.reserve(need, clue::bridge_budget(h)))) return rc;
    if ((rc = h->stage.reserve(8 * (size_t)(E + 1) + 4 * (size_t)nch))) return rc;
    auto P = [&](int s) { return h->arena_bridge.ptr(s); };
    cudaStream_t s = h->stream;
    memcpy(h->stage.p, off, 8 * (size_t)(E + 1));
    int32_t* cev = reinterpret_cast<int32_t*>(static_cast<char*>(h->stage.p) + 8 * (size_t)(E + 1));
    clue::chunk_events(E, off, nch, cev);
    if ((e = cudaMemcpyAsync(P(clue::B_OFF), h->stage.p, 8 * (size_t)(E + 1), cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(P(clue::B_CEV), cev, 4 * (size_t)nch, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(P(clue::B_COUNT), 0, 4 * (size_t)E, s)))
      return cuda_error(e, "bridge set-up");
    if (N > 0)
      clue::k_bridge_count<<<nch, clue::kBridgeThreads, 0, s>>>(N, static_cast<const int64_t*>(P(clue::B_OFF)),
                                                                  static_cast<const int32_t*>(P(clue::B_CEV)),
                                                                  isSeed, static_cast<int32_t*>(P(clue::B_COUNT)));
    if ((e = cudaGetLastError())) return cuda_error(e, "k_bridge_count");
    std::vector<int32_t> counts(E);
    if ((e = cudaMemcpyAsync(counts.data(), P(clue::B_COUNT), 4 * (size_t)E, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_error(e, "bridge counts");
    for (int32_t i = 0; i < E; ++i) cluster_offsets[i + 1] = cluster_offsets[i] + counts[i];
    return CLUE_OK;
  });
}

int clue_bridge_build(clue_handle* hh, const clue_bridge_params* p, int32_t E, const int64_t* off, const float* x,
                      const float* y, const int32_t* layer, const float* weight, const int32_t* isSeed,
                      const int32_t* clusterIndex, const int64_t* coff, const clue_layer_clusters* out) {
  return clue::guarded([&]() -> int {
    if (!hh || !p || !out) return set_error(CLUE_EINVAL, "NULL argument");
    int rc = clue::check_offsets(E, off, "event_offsets");
    if (rc) return rc;
    if ((rc = clue::check_offsets(E, coff, "cluster_offsets"))) return rc;
    if (p->n_layers < 1 || !p->layer_z) return set_error(CLUE_EINVAL, "bridge needs n_layers >= 1 and a z table");
    if (E == 0) return CLUE_OK;
    const int64_t N = off[E], C = coff[E];
    if (N > 0 && (!x || !y || !layer || !weight || !isSeed || !clusterIndex))
      return set_error(CLUE_EINVAL, "NULL input array");
    const void* outs[10] = {out->x, out->y, out->z, out->eta, out->phi, out->r_over_absz, out->radius,
                            out->layer, out->energy, out->isSilicon};
    if (C > 0)
      for (auto q : outs)
        if (!q) return set_error(CLUE_EINVAL, "NULL output array");
    Handle* h = reinterpret_cast<Handle*>(hh);
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    if ((rc = h->wait_previous())) return rc;
    std::vector<size_t> need(clue::B_SLOTS, 0);
    need[clue::B_OFF] = need[clue::B_COFF] = 8 * (size_t)(E + 1);
    need[clue::B_COUNT] = 4 * (size_t)E;
    need[clue::B_ACC] = 24 * (size_t)std::max<int64_t>(C, 1);
    need[clue::B_SEED] = 4 * (size_t)std::max<int64_t>(C, 1);
    need[clue::B_LZ] = 4 * (size_t)p->n_layers;
    need[clue::B_FLAGS] = 4 * clue::kFlagCount;
    const int nch = clue::chunks_for(N);
    need[clue::B_CEV] = 4 * (size_t)std::max(nch, 1);
    if ((rc = h->arena_bridge.reserve(need, clue::bridge_budget(h)))) return rc;
    const size_t stage_bytes = 16 * (size_t)(E + 1) + 4 * (size_t)p->n_layers + 4 * (size_t)nch;
    if ((rc = h->stage.reserve(stage_bytes))) return rc;
    if ((rc = h->flags_host.reserve(4 * clue::kFlagCount))) return rc;
    auto P = [&](int s) { return h->arena_bridge.ptr(s); };
    char* st = static_cast<char*>(h->stage.p);
    memcpy(st, off, 8 * (size_t)(E + 1));
    memcpy(st + 8 * (size_t)(E + 1), coff, 8 * (size_t)(E + 1));
    memcpy(st + 16 * (size_t)(E + 1), p->layer_z, 4 * (size_t)p->n_layers);
    int32_t* cev = reinterpret_cast<int32_t*>(st + 16 * (size_t)(E + 1) + 4 * (size_t)p->n_layers);
    clue::chunk_events(E, off, nch, cev);
    cudaStream_t s = h->stream;
    if ((e = cudaMemcpyAsync(P(clue::B_OFF), st, 8 * (size_t)(E + 1), cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(P(clue::B_COFF), st + 8 * (size_t)(E + 1), 8 * (size_t)(E + 1), cudaMemcpyHostToDevice,
                             s)) ||
        (e = cudaMemcpyAsync(P(clue::B_LZ), st + 16 * (size_t)(E + 1), 4 * (size_t)p->n_layers,
                             cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(P(clue::B_ACC), 0, 24 * (size_t)std::max<int64_t>(C, 1), s)) ||
        (e = cudaMemsetAsync(P(clue::B_SEED), 0, 4 * (size_t)std::max<int64_t>(C, 1), s)) ||
        (e = cudaMemsetAsync(P(clue::B_FLAGS), 0, 4 * clue::kFlagCount, s)) ||
        (e = cudaMemcpyAsync(P(clue::B_CEV), cev, 4 * (size_t)nch, cudaMemcpyHostToDevice, s)))
      return cuda_error(e, "bridge set-up");
    int32_t* flags = static_cast<int32_t*>(P(clue::B_FLAGS));
    auto* acc = static_cast<unsigned long long*>(P(clue::B_ACC));
    auto* seed_of = static_cast<int32_t*>(P(clue::B_SEED));
    if (N > 0)
      clue::k_bridge_accumulate<<<nch, clue::kBridgeThreads, 0, s>>>(
          N, static_cast<const int64_t*>(P(clue::B_OFF)), static_cast<const int32_t*>(P(clue::B_CEV)),
          static_cast<const int64_t*>(P(clue::B_COFF)), x, y, weight, isSeed, clusterIndex, acc, seed_of, flags);
    if ((e = cudaGetLastError())) return cuda_error(e, "k_bridge_accumulate");
    if (C > 0)
      clue::k_bridge_finalize<<<clue::grid_for(C), 256, 0, s>>>(C, acc, seed_of, x, y, layer,
                                                                 static_cast<const float*>(P(clue::B_LZ)),
                                                                 p->n_layers, p->radius, p->isSilicon, *out, flags);
    if ((e = cudaGetLastError())) return cuda_error(e, "k_bridge_finalize");
    if ((e = cudaMemcpyAsync(h->flags_host.p, flags, 4 * clue::kFlagCount, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_error(e, "bridge");
    int32_t* fh = static_cast<int32_t*>(h->flags_host.p);
    const int32_t err = fh[clue::kFlagError];
    fh[clue::kFlagError] = 0;
    if (err == 1) return set_error(CLUE_EINVAL, "a clusterIndex is not below its event's cluster count");
    if (err == 2) return set_error(CLUE_EINVAL, "a layer cluster's layer is outside [0, %d)", p->n_layers);
    return CLUE_OK;
  });
}

}  // extern "C"
