// CLUE3D on GB300: the SoA tracksterizer stages of
// src/serial/plugin-CLUETracksterizer/CLUE3DAlgoKernels.h re-designed for
// batches of events.
//
// Layout: per event, the layer clusters are counting-sorted by their flat
// tile key  key = layer*4284 + phiBin + 126*etaBin  (the reference's tiles
// are one contiguous array over layers, so an eta row of 34 lands in the next
// layer's row 0, and phiBin may be 126; both are reproduced).  A "row" is
// key/126 (one (layer, eta) line of 126 phi bins); inside a row entries are
// ordered by (phi bin, index), which is the reference's visiting order for
// a phi window that does not wrap.  A wrapping window is visited as its two
// arcs in the reference's order.
//
// Stages (one launch each, flattened over all events of the batch):
//   k3_key        flat key per cluster; clusters per (event, row)
//   k3_row_scan   per event: first position of each row
//   k3_scatter    place clusters into their rows (arbitrary order)
//   k3_row_sort   order each row by (phi bin, index)
//   k3_density    KernelCalculateDensitySoA (:26-150)
//   k3_nh         KernelComputeDistanceToHigherSoA (:286-392)
//   k3_flags      seeds, outliers, parent pointers (:509-560)
//   k3_finish     per event: trackster ids by seed rank, pointer jumping
//                 along nearestHigher, labels (:564-577)
// Float arithmetic uses explicit _rn intrinsics in the reference's operation
// order; phiBin's product is in double, as in TICLLayerTile.h:28-34.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>

#include "clue_internal.h"

namespace clue {
namespace {

constexpr int kEtaBins = 34;
constexpr int kPhiBins = 126;
constexpr int kBins = kEtaBins * kPhiBins;

__device__ __forceinline__ int event_of(const int64_t* off, int n_events, int64_t i) {
  int lo = 0, hi = n_events;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// reco::reduceRange for float (src/serial/DataFormats/Math/deltaPhi.h:16-23)
__device__ __forceinline__ float reduce_range(float x, const Params3D& P) {
  if (fabsf(x) <= P.pi_f) return x;
  const float n = roundf(__fmul_rn(x, P.o2pi));
  return __fsub_rn(x, __fmul_rn(n, P.twopi_f));
}

// TICLLayerTileT::etaBin (src/serial/DataFormats/TICLLayerTile.h:19-26)
__device__ __forceinline__ int eta_bin(float eta, const Params3D& P) {
  const int b = __float2int_rz(__fmul_rn(__fsub_rn(fabsf(eta), 1.5f), P.eta_r));
  return min(max(b, 0), kEtaBins - 1);
}

// TICLLayerTileT::phiBin (TICLLayerTile.h:28-34): (normPhi + M_PI) * r in double.
// A NaN (phi NaN or +-inf, which reduce to NaN) takes bin 0: the reference's
// int conversion is undefined there, 0 on the aarch64 host, and the device's
// conversion would give INT_MIN.
__device__ __forceinline__ int phi_bin(float phi, const Params3D& P) {
  const float norm = reduce_range(phi, P);
  if (norm != norm) return 0;
  return __double2int_rz(__dmul_rn(__dadd_rn((double)norm, 3.14159265358979323846), (double)P.phi_r));
}

// The reference's layer window (CLUE3DAlgoKernels.h:49-58 density, :308-317
// nearest higher; the upper side starts one layer later there).
__device__ __forceinline__ void layer_window(int layer, int sib, int n_layers, int upper_shift, int* lo, int* hi) {
  const int last = n_layers / 2;
  int mx = 2 * last - 1, mn = 0;
  if (layer < last) {
    mn = max(layer - sib, mn);
    mx = min(layer + sib, last - 1);
  } else {
    mn = max(layer - sib, last + upper_shift);
    mx = min(layer + sib, mx);
  }
  *lo = mn;
  *hi = mx;
}

// Row of a flat key; clusters rejected by k3_key (key -1) go to the
// event's last row, which no search visits.
__device__ __forceinline__ int row_of(int k, int n_rows) { return k >= 0 ? k / kPhiBins : n_rows - 1; }

__global__ void k3_key(Batch3D b, Params3D P) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int row = -1, e = 0;
  if (i < b.n_points) {
    e = event_of(b.offsets, b.n_events, i);
    const int l = b.layer[i];
    const int pb = phi_bin(b.phi[i], P);
    int k = -1;
    if (l < 0 || l >= P.n_layers) {
      atomicExch(&b.flags[kFlagError], 1);
    } else if (pb < 0 || pb > kPhiBins) {
      atomicExch(&b.flags[kFlagError], 2);
    } else {
      k = l * kBins + pb + eta_bin(b.eta[i], P) * kPhiBins;
    }
    b.key[i] = k;
    row = row_of(k, b.n_rows);
  }
  const int gkey = row >= 0 ? e * b.n_rows + row : -1;
  const unsigned mask = __match_any_sync(0xffffffffu, gkey);
  if (gkey >= 0 && (threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd(&b.row_cnt[gkey], __popc(mask));
}

// One block per event: exclusive scan of its rows.
__global__ void __launch_bounds__(256) k3_row_scan(Batch3D b) {
  const int e = blockIdx.x;
  const int R = b.n_rows;
  const int per = (R + 255) / 256;
  const int beg = min((int)threadIdx.x * per, R), end = min(beg + per, R);
  const int32_t* cnt = b.row_cnt + (int64_t)e * R;
  int sum = 0;
  for (int r = beg; r < end; ++r) sum += cnt[r];
  __shared__ int s_w[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += s_w[w];
  int run = (int)b.offsets[e] + before + x - sum;
  for (int r = beg; r < end; ++r) {
    b.row_start[(int64_t)e * R + r] = run;
    b.cursor[(int64_t)e * R + r] = run;
    run += cnt[r];
  }
  if (e == b.n_events - 1 && threadIdx.x == 255) b.row_start[(int64_t)b.n_events * R] = (int)b.offsets[b.n_events];
}

__global__ void k3_scatter(Batch3D b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int gkey = -1, e = 0, k = -1;
  if (i < b.n_points) {
    e = event_of(b.offsets, b.n_events, i);
    k = b.key[i];
    gkey = e * b.n_rows + row_of(k, b.n_rows);
  }
  const unsigned mask = __match_any_sync(0xffffffffu, gkey);
  const int leader = __ffs(mask) - 1;
  const int lane = threadIdx.x & 31;
  int pos = 0;
  if (gkey >= 0 && lane == leader) pos = atomicAdd(&b.cursor[gkey], __popc(mask));
  pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(mask & ((1u << lane) - 1u));
  if (gkey >= 0) {
    b.tmp[pos] = (int32_t)(i - b.offsets[e]);  // event-local index
    b.par[pos] = k >= 0 ? k % kPhiBins : 0;     // phi column
  }
}

// Each entry's rank inside its row by (column, index) gives its final slot.
__global__ void k3_row_sort(Batch3D b) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= b.n_points) return;
  const int e = event_of(b.offsets, b.n_events, p);
  const int idx = b.tmp[p], col = b.par[p];
  const int k = b.key[b.offsets[e] + idx];
  const int64_t r = (int64_t)e * b.n_rows + row_of(k, b.n_rows);
  const int s = b.row_start[r], t = b.row_start[r + 1];
  int rank = 0;
  for (int q = s; q < t; ++q) {
    const int c2 = b.par[q], i2 = b.tmp[q];
    rank += (c2 < col) || (c2 == col && i2 < idx);
  }
  b.sorted[s + rank] = idx;
  b.scol[s + rank] = col;
  // what the searches read of a candidate, in sorted order: a run of a row's
  // entries is then one contiguous stretch of 16-byte records (rho follows
  // from the density search)
  const int64_t gi = b.offsets[e] + idx;
  b.cand[s + rank] = make_float4(b.roa[gi], b.phi[gi], b.energy[gi], 0.f);
  // occupancy of the row's phi columns; bit 127 marks a column held twice
  unsigned long long* m = b.row_mask + 2 * r;
  const unsigned long long bit = 1ull << (col & 63);
  if (atomicOr(m + (col >> 6), bit) & bit) atomicOr(m + 1, 1ull << 63);
}

// Visits the entries of one row whose phi column lies in the window
// [p0, p1] (p0 may be negative, p1 may exceed 125), in the reference's
// order: iphi_it = p0..p1 mapped modulo 126.
// Entries of a row whose phi column lies in [a, c] (0 <= a <= c <= 125) are
// one run of the row (entries are sorted by column): its first position and
// length, from the column-occupancy mask, when no column repeats.
__device__ __forceinline__ int bits_below(unsigned long long m0, unsigned long long m1, int p) {
  // set bits of columns < p (0 <= p <= 126)
  if (p <= 0) return 0;
  if (p < 64) return __popcll(m0 & ((1ull << p) - 1));
  return __popcll(m0) + __popcll(m1 & ((1ull << (p - 64)) - 1));
}

// visit_row() for row r through its occupancy mask: the row start is read
// only when the window holds an entry, and the row is not scanned.
template <class F>
__device__ __forceinline__ void visit_row_masked(const Batch3D& b, int64_t r, int p0, int p1, F&& f) {
  const unsigned long long m0 = b.row_mask[2 * r], m1 = b.row_mask[2 * r + 1];
  if (m1 >> 63) {  // a column holds several entries: walk the row
    visit_row(b, b.row_start[r], b.row_start[r + 1], p0, p1, f);
    return;
  }
  int a0, c0, a1 = 0, c1 = -1;  // first run [a0, c0], then [a1, c1] (wrapping windows)
  if (p0 >= 0 && p1 < kPhiBins) {
    a0 = p0; c0 = p1;
  } else if (p0 < 0) {
    a0 = p0 + kPhiBins; c0 = kPhiBins - 1; a1 = 0; c1 = p1;
  } else {
    a0 = p0; c0 = kPhiBins - 1; a1 = 0; c1 = p1 - kPhiBins;
  }
  const int lo0 = bits_below(m0, m1, a0), n0 = bits_below(m0, m1, c0 + 1) - lo0;
  const int n1 = c1 >= a1 ? bits_below(m0, m1, c1 + 1) : 0;  // the second run starts at column 0
  if (n0 + n1 == 0) return;
  const int s = b.row_start[r];
  for (int q = s + lo0; q < s + lo0 + n0; ++q) f(q);
  for (int q = s; q < s + n1; ++q) f(q);
}

template <class F>
__device__ __forceinline__ void visit_row(const Batch3D& b, int s, int t, int p0, int p1, F&& f) {
  if (p0 >= 0 && p1 < kPhiBins) {
    for (int q = s; q < t; ++q) {
      const int c = b.scol[q];
      if (c > p1) break;
      if (c >= p0) f(q);
    }
    return;
  }
  int a0, a1, c0, c1;  // first arc [a0, a1], then [c0, c1]
  if (p0 < 0) {
    a0 = p0 + kPhiBins; a1 = kPhiBins - 1; c0 = 0; c1 = p1;
  } else {
    a0 = p0; a1 = kPhiBins - 1; c0 = 0; c1 = p1 - kPhiBins;
  }
  for (int q = s; q < t; ++q) {
    const int c = b.scol[q];
    if (c >= a0 && c <= a1) f(q);
  }
  for (int q = s; q < t; ++q) {
    const int c = b.scol[q];
    if (c > c1) break;
    if (c >= c0) f(q);
  }
}

// 40 registers (6 blocks per SM): 4.76 ms against 5.26 ms at the compiler's
// 56 on the 1,000-event batch
__global__ void __launch_bounds__(256, 6) k3_density(Batch3D b, Params3D P) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= b.n_points) return;
  const int e = event_of(b.offsets, b.n_events, p);
  const int64_t es = b.offsets[e];
  const int i = b.sorted[p];  // clusters processed in tile order for locality
  const int64_t gi = es + i;
  const int li = b.layer[gi];
  if (b.key[gi] < 0) return;
  int lo, hi;
  layer_window(li, P.dens_sib, P.n_layers, 0, &lo, &hi);
  const float eta_i = b.eta[gi], phi_i = b.phi[gi], zi = b.z[gi];
  const int eb = eta_bin(eta_i, P), pb = phi_bin(phi_i, P);
  const float thr = b.sil[gi] ? P.dens_thr : __fmul_rn(b.radius[gi], b.radius[gi]);
  const float r0 = __fmul_rn(b.roa[gi], zi);
  const int64_t rbase = (int64_t)e * b.n_rows;
  float rho = 0.f;
  for (int cl = lo; cl <= hi; ++cl) {
    const bool same = (cl == li);
    const float coef = __fmul_rn(P.kdf, (same && !P.dens_same) ? 0.f : 1.f);
    const int e0 = max(eb - 2, 0), e1 = min(eb + 2, kEtaBins);
    for (int ie = e0; ie <= e1; ++ie) {
      const int64_t r = rbase + (int64_t)cl * kEtaBins + ie;
      visit_row_masked(b, r, pb - 2, pb + 2, [&](int q) {
        const float4 cj = b.cand[q];  // {roa, phi, energy, -}; q == p is the cluster itself
        const float r1 = __fmul_rn(cj.x, zi);
        const float dphi = reduce_range(__fsub_rn(phi_i, cj.y), P);
        const float d0 = __fsub_rn(r0, r1);
        const float a = __fmul_rn(d0, d0);
        const float c = __fmul_rn(__fmul_rn(__fmul_rn(r1, r1), dphi), dphi);
        if (__fadd_rn(a, c) < thr) rho = __fadd_rn(rho, __fmul_rn((q == p) ? 1.f : coef, cj.z));
      });
    }
  }
  b.rho[gi] = rho;
  reinterpret_cast<float*>(b.cand)[4 * p + 3] = rho;
}

// 40 registers (6 blocks per SM), as k3_density: 4.76 -> 4.58 ms per batch
__global__ void __launch_bounds__(256, 6) k3_nh(Batch3D b, Params3D P) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= b.n_points) return;
  const int e = event_of(b.offsets, b.n_events, p);
  const int64_t es = b.offsets[e];
  const int i = b.sorted[p];
  const int64_t gi = es + i;
  const int li = b.layer[gi];
  if (b.key[gi] < 0) return;
  int lo, hi;
  layer_window(li, P.nh_sib, P.n_layers, 1, &lo, &hi);
  const float eta_i = b.eta[gi], phi_i = b.phi[gi], zi = b.z[gi], rho_i = b.rho[gi];
  const int eb = eta_bin(eta_i, P), pb = phi_bin(phi_i, P);
  const float r0 = __fmul_rn(b.roa[gi], zi);
  const int64_t rbase = (int64_t)e * b.n_rows;
  float best = FLT_MAX, best_t = FLT_MAX;
  int best_l = INT_MAX, nl = -1, ni = -1;
  for (int cl = lo; cl <= hi; ++cl) {
    if (!P.nh_same && cl == li) continue;
    const int e0 = max(eb - 1, 0), e1 = min(eb + 1, kEtaBins);
    for (int ie = e0; ie <= e1; ++ie) {
      const int64_t r = rbase + (int64_t)cl * kEtaBins + ie;
      visit_row_masked(b, r, pb - 1, pb + 1, [&](int q) {
        const float4 cj = b.cand[q];  // {roa, phi, energy, rho}
        const float r1 = __fmul_rn(cj.x, zi);
        const float dphi = reduce_range(__fsub_rn(phi_i, cj.y), P);
        const float d0 = __fsub_rn(r0, r1);
        const float d = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(__fmul_rn(__fmul_rn(r1, r1), dphi), dphi));
        if (cj.w > rho_i && d <= best) {  // "<=": the last candidate wins a tie
          best = d;
          best_t = __fsqrt_rn(d);
          best_l = abs(cl - li);
          nl = cl;
          ni = b.sorted[q];
        }
      });
    }
  }
  if (best != FLT_MAX) {
    b.delta_t[gi] = best_t;
    b.delta_l[gi] = best_l;
    b.nh_l[gi] = nl;
    b.nh_i[gi] = ni;
  } else {
    b.delta_t[gi] = FLT_MAX;
    b.delta_l[gi] = INT_MAX;
    b.nh_l[gi] = -1;
    b.nh_i[gi] = -1;
  }
}

// Seeds and outliers (CLUE3DAlgoKernels.h:521-560).  par: nearest higher for
// followers, -2 for seeds, -3 for other roots.
__global__ void k3_flags(Batch3D b, Params3D P) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= b.n_points) return;
  if (b.key[i] < 0) {
    b.seed[i] = 0;
    b.par[i] = -3;
    return;
  }
  const float dt = b.delta_t[i], r = b.rho[i];
  const float dxy = b.sil[i] ? P.crit_xy : b.radius[i];
  const bool seed = (dt > dxy || __int2float_rn(b.delta_l[i]) > P.crit_z) && (r >= P.crit_rho) &&
                    (__fdiv_rn(b.energy[i], r) > P.crit_self);
  const bool outlier = (dt > P.out_thr) && (r < P.crit_rho);
  b.seed[i] = seed ? 1 : 0;
  b.par[i] = seed ? -2 : ((!outlier && b.nh_l[i] >= 0) ? b.nh_i[i] : -3);
}

// One block per event: trackster ids by seed rank in index order, then
// pointer jumping along nearestHigher (replaces the LIFO propagation), then
// labels.  par holds event-local indices.
__global__ void __launch_bounds__(512) k3_finish(Batch3D b) {
  const int e = blockIdx.x;
  const int64_t es = b.offsets[e];
  const int n = (int)(b.offsets[e + 1] - es);
  int32_t* par = b.par + es;
  int32_t* ti = b.ti + es;
  const int32_t* seed = b.seed + es;
  __shared__ int s_w[16];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 512) {
    const int i = base + threadIdx.x;
    const int f = (i < n) ? seed[i] : 0;
    int x = f;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    int before = s_base;
    for (int w = 0; w < warp; ++w) before += s_w[w];
    if (i < n) ti[i] = f ? before + x - 1 : -1;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < 16; ++w) tot += s_w[w];
      s_base += tot;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) b.ev_seeds[e] = s_base;
  for (;;) {
    int changed = 0;
    for (int i = threadIdx.x; i < n; i += 512) {
      const int p = par[i];
      if (p >= 0) {
        const int pp = par[p];
        if (pp >= 0) {
          par[i] = pp;
          changed = 1;
        }
      }
    }
    if (!__syncthreads_or(changed)) break;
  }
  for (int i = threadIdx.x; i < n; i += 512) {
    if (seed[i]) continue;
    const int p = par[i];
    ti[i] = (p >= 0 && par[p] == -2) ? ti[p] : -1;
  }
}

}  // namespace

cudaError_t launch_clue3d(const Batch3D& b, const Params3D& p, cudaStream_t s) {
  if (b.n_events <= 0 || b.n_points <= 0) return cudaSuccess;
  cudaError_t err = cudaMemsetAsync(b.row_cnt, 0, sizeof(int32_t) * (size_t)b.n_events * b.n_rows, s);
  if (err != cudaSuccess) return err;
  err = cudaMemsetAsync(b.row_mask, 0, 16 * (size_t)b.n_events * b.n_rows, s);
  if (err != cudaSuccess) return err;
  const int T = 256;
  const int grid = (int)((b.n_points + T - 1) / T);
  {
    NvtxRange r("clue3d/key");
    k3_key<<<grid, T, 0, s>>>(b, p);
  }
  {
    NvtxRange r("clue3d/row_scan");
    k3_row_scan<<<b.n_events, 256, 0, s>>>(b);
  }
  {
    NvtxRange r("clue3d/scatter");
    k3_scatter<<<grid, T, 0, s>>>(b);
  }
  {
    NvtxRange r("clue3d/row_sort");
    k3_row_sort<<<grid, T, 0, s>>>(b);
  }
  {
    NvtxRange r("clue3d/density");
    k3_density<<<grid, T, 0, s>>>(b, p);
  }
  {
    NvtxRange r("clue3d/nearest_higher");
    k3_nh<<<grid, T, 0, s>>>(b, p);
  }
  {
    NvtxRange r("clue3d/flags");
    k3_flags<<<grid, T, 0, s>>>(b, p);
  }
  {
    NvtxRange r("clue3d/finish");
    k3_finish<<<b.n_events, 512, 0, s>>>(b);
  }
  return cudaGetLastError();
}

}  // namespace clue
