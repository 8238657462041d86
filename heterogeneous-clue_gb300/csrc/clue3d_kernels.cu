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
//   k3_key        flat key per cluster; clusters per (event, row) and each
//                 cluster's arrival slot in its row
//   k3_row_scan   per event: first position of each row
//   k3_scatter    place clusters into their rows (arrival order) with their
//                 candidate and query records; row occupancy and repeat masks
//   k3_row_sort   order each row by (phi bin, index): a counting sort by
//                 column through the mask, or a count where a column repeats
//   k3_search<true>   KernelCalculateDensitySoA (:26-150), one block per
//                     (event, slab of layers) with the slab's rows staged
//   k3_search<false>  KernelComputeDistanceToHigherSoA (:286-392), likewise,
//                     then seeds, outliers and parent pointers (:509-560)
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

// Event of cluster i: from the event of its 256-cluster block's first
// cluster, forward past the events that end at or before i.
__device__ __forceinline__ int event_of_blk(const Batch3D& b, int64_t i) {
  int e = b.blk_ev[i >> 8];
  while (b.offsets[e + 1] <= i) ++e;
  return e;
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
    e = event_of_blk(b, i);
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
    if (k < 0) b.seed[i] = -1;  // not searched: k3_finish makes it a root of its own
    row = row_of(k, b.n_rows);
  }
  const int gkey = row >= 0 ? e * b.n_rows + row : -1;
  const unsigned mask = __match_any_sync(0xffffffffu, gkey);
  const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
  int old = 0;
  if (gkey >= 0 && lane == leader) old = atomicAdd(&b.row_cnt[gkey], __popc(mask));
  old = __shfl_sync(0xffffffffu, old, leader);
  if (gkey >= 0) b.arr[i] = old + __popc(mask & ((1u << lane) - 1u));
}

// Entries of a row whose phi column lies in [a, c] (0 <= a <= c <= 125) are
// one run of the row (entries are sorted by column): its first position and
// length, from the column-occupancy mask, when no column repeats.
__device__ __forceinline__ int bits_below(unsigned long long m0, unsigned long long m1, int p) {
  // set bits of columns < p (0 <= p <= 126)
  if (p <= 0) return 0;
  if (p < 64) return __popcll(m0 & ((1ull << p) - 1));
  return __popcll(m0) + __popcll(m1 & ((1ull << (p - 64)) - 1));
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
    run += cnt[r];
  }
  if (e == b.n_events - 1 && threadIdx.x == 255) b.row_start[(int64_t)b.n_events * R] = (int)b.offsets[b.n_events];
}

// Each cluster to its arrival slot in its row, with everything the row sort
// and the searches need of it, read here in input order (coalesced): its
// event-local index, phi column and row; its 16-byte candidate record {roa,
// phi, energy, rho} (rho added by the density search); its 16-byte query
// record {z, roa * z, density threshold, layer | etaBin << 11 | phiBin << 17 |
// isSilicon << 24}.
// The cluster also goes into its row's 128-bit phi-column occupancy mask;
// bit 127 marks a column held twice.
__global__ void k3_scatter(Batch3D b, Params3D P) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= b.n_points) return;
  const int e = event_of_blk(b, i);
  const int k = b.key[i];
  const int row = row_of(k, b.n_rows);
  const int64_t r = (int64_t)e * b.n_rows + row;
  const int pos = b.row_start[r] + b.arr[i];
  const int col = k >= 0 ? k % kPhiBins : 0;
  b.tmp[pos] = (int32_t)(i - b.offsets[e]);
  b.par[pos] = col | (row << 7);
  const float roa = b.roa[i];
  b.tcand[pos] = make_float4(roa, b.phi[i], b.energy[i], 0.f);
  if (k >= 0) {
    const float zi = b.z[i];
    const float thr = b.sil[i] ? P.dens_thr : __fmul_rn(b.radius[i], b.radius[i]);
    // the phi bin from the key (key = layer * 4284 + phiBin + 126 * etaBin,
    // phiBin up to 126), without k3_key's double-precision product again
    const int li = b.layer[i], eb = eta_bin(b.eta[i], P);
    const int pbin = k - li * kBins - eb * kPhiBins;
    const int bins = li | (eb << 11) | (pbin << 17) | ((b.sil[i] ? 1 : 0) << 24);
    b.tqrec[pos] = make_float4(zi, __fmul_rn(roa, zi), thr, __int_as_float(bins));
  } else {
    b.tqrec[pos] = make_float4(0.f, 0.f, 0.f, 0.f);  // the junk row's entries are never queried
  }
  unsigned long long* m = b.row_mask + 2 * r;
  const unsigned long long bit = 1ull << (col & 63);
  if (atomicOr(m + (col >> 6), bit) & bit) {
    atomicOr(m + 1, 1ull << 63);
    // a second entry in the column: the column's bit in the repeat mask; a
    // third: bit 127 of the repeat mask
    unsigned long long* rp = b.row_rep + 2 * r;
    if (atomicOr(rp + (col >> 6), bit) & bit) atomicOr(rp + 1, 1ull << 63);
  }
}

// Each entry's rank inside its row by (column, index) gives its final slot:
// a counting sort by column through the occupancy mask (the entries in lower
// columns are the mask's set bits below the entry's column) when no column
// repeats, a count over the row otherwise.  One thread per scattered entry;
// its records move within the row's range.
__global__ void k3_row_sort(Batch3D b) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= b.n_points) return;
  const int e = event_of_blk(b, p);
  const int idx = b.tmp[p], cr = b.par[p];
  const int col = cr & 127;
  const int64_t r = (int64_t)e * b.n_rows + (cr >> 7);
  const int s = b.row_start[r];
  const ulonglong2 m = reinterpret_cast<const ulonglong2*>(b.row_mask)[r];
  int rank;
  if (!(m.y >> 63)) {
    rank = bits_below(m.x, m.y, col);
  } else {
    const int t = b.row_start[r + 1];
    rank = 0;
    for (int q = s; q < t; ++q) {
      const int c2 = b.par[q] & 127, i2 = b.tmp[q];
      rank += (c2 < col) || (c2 == col && i2 < idx);
    }
  }
  const int f = s + rank;
  b.sorted[f] = idx;
  b.scol[f] = col;
  b.cand[f] = b.tcand[p];
  b.qrec[f] = b.tqrec[p];
}

// The rows of one event as the searches see them: the whole event in global
// memory, or a staged copy of a range of rows in shared memory.  Positions
// are sorted positions (global, or relative to the first staged entry).
struct RowsGlobal {
  const unsigned long long* mask;  // 2 words per row of the event
  const int32_t* rstart;           // first sorted position of each row of the event
  const float4* cand;
  const int32_t* scol;
  __device__ __forceinline__ unsigned long long m0(int r) const { return mask[2 * r]; }
  __device__ __forceinline__ unsigned long long m1(int r) const { return mask[2 * r + 1]; }
  __device__ __forceinline__ int start(int r) const { return rstart[r]; }
  __device__ __forceinline__ float4 rec(int q) const { return cand[q]; }
  __device__ __forceinline__ int col(int q) const { return scol[q]; }
};

struct RowsStaged {
  const unsigned long long* mask;  // 2 words per staged row
  const unsigned long long* rmask; // 2 words per staged row: columns holding two entries; bit 127: three or more
  const int32_t* rstart;           // relative to the first staged entry
  const float4* cand;
  const uint8_t* scol;
  int row_lo;  // first staged row
  __device__ __forceinline__ unsigned long long m0(int r) const { return mask[2 * (r - row_lo)]; }
  __device__ __forceinline__ unsigned long long m1(int r) const { return mask[2 * (r - row_lo) + 1]; }
  __device__ __forceinline__ ulonglong2 mm(int r) const {
    return reinterpret_cast<const ulonglong2*>(mask)[r - row_lo];
  }
  __device__ __forceinline__ ulonglong2 rep(int r) const {
    return reinterpret_cast<const ulonglong2*>(rmask)[r - row_lo];
  }
  __device__ __forceinline__ int start(int r) const { return rstart[r - row_lo]; }
  __device__ __forceinline__ float4 rec(int q) const { return cand[q]; }
  __device__ __forceinline__ int col(int q) const { return scol[q]; }
};

// Visits the entries of rows [s, t) whose phi column lies in the window
// [p0, p1] (p0 may be negative, p1 may exceed 125), in the reference's
// order: iphi_it = p0..p1 mapped modulo 126.
template <class V, class F>
__device__ __forceinline__ void visit_row(const V& v, int s, int t, int p0, int p1, F&& f) {
  if (p0 >= 0 && p1 < kPhiBins) {
    for (int q = s; q < t; ++q) {
      const int c = v.col(q);
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
    const int c = v.col(q);
    if (c >= a0 && c <= a1) f(q);
  }
  for (int q = s; q < t; ++q) {
    const int c = v.col(q);
    if (c > c1) break;
    if (c >= c0) f(q);
  }
}

// Phi columns of the window [pb - d, pb + d] modulo 126 as a 126-bit mask
// (the reference's iphi = iphi_it mod nPhiBins, CLUE3DAlgoKernels.h:80-84).
struct ColMask {
  unsigned long long w0 = 0, w1 = 0;
  // columns [lo, lo + n), 0 <= n <= 5, lo + n <= 126
  __device__ __forceinline__ void run(int lo, int n) {
    const unsigned long long r = (1ull << n) - 1;
    if (lo >= 64) {
      w1 |= r << (lo - 64);
    } else {
      w0 |= r << lo;
      if (lo + n > 64) w1 |= r >> (64 - lo);
    }
  }
  __device__ __forceinline__ ColMask(int pb, int d) {  // 0 <= pb <= 126, d <= 2
    const int a = pb - d, c = pb + d;
    if (a < 0) {
      run(a + kPhiBins, -a);
      run(0, c + 1);
    } else if (c >= kPhiBins) {
      run(a, kPhiBins - a);
      run(0, c - kPhiBins + 1);
    } else {
      run(a, 2 * d + 1);
    }
  }
};

// visit_row() for row r through its occupancy mask: a row with no entry in
// the window's columns is skipped on the mask alone, the row start is read
// only when the window holds an entry, and the row is not scanned.
template <class V, class F>
__device__ __forceinline__ void visit_row_masked(const V& v, int r, const ColMask& wm, int p0, int p1, F&& f) {
  const unsigned long long m0 = v.m0(r), m1 = v.m1(r);
  // bit 127 of m1 marks a repeated column; the window never holds column 127
  if (((m0 & wm.w0) | (m1 & wm.w1)) == 0) return;
  if (m1 >> 63) {  // a column holds several entries: walk the row
    visit_row(v, v.start(r), v.start(r + 1), p0, p1, f);
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
  const int s = v.start(r);
  for (int q = s + lo0; q < s + lo0 + n0; ++q) f(q);
  for (int q = s; q < s + n1; ++q) f(q);
}

// Rows of a query's window that hold an entry in its phi columns, as bits
// (cl - lo) * 8 + (ie - e0) of a 64-bit word: ascending bit order is the
// reference's visiting order (layers outer, eta rows inner).  Reading every
// row's mask in one uniform pass and then visiting only the rows whose bit is
// set keeps the lanes of a warp together: otherwise each of the ~25 rows would
// send the few lanes with an entry down the visit while the others wait.
// Windows of more than 8 layers or 5 eta rows return false (the caller loops
// directly).
template <class V>
__device__ __forceinline__ bool live_rows(const V& v, int lo, int hi, int skip, int e0, int e1, const ColMask& wm,
                                          unsigned long long* live) {
  if (hi - lo >= 8 || e1 - e0 >= 5) return false;
  unsigned long long m = 0;
  const int ne = e1 - e0;
  for (int cl = lo; cl <= hi; ++cl) {
    if (cl == skip) continue;
    // a layer's (at most five) window rows are consecutive: their masks are
    // read together and their bits set with one shift
    const int r0 = cl * kEtaBins + e0;
    unsigned bits = 0;
#pragma unroll
    for (int de = 0; de < 5; ++de) {
      if (de <= ne) {
        const ulonglong2 rm = v.mm(r0 + de);
        bits |= (((rm.x & wm.w0) | (rm.y & wm.w1)) != 0ull ? 1u : 0u) << de;
      }
    }
    m |= (unsigned long long)bits << ((cl - lo) * 8);
  }
  *live = m;
  return true;
}

// What a search needs of its query cluster.
struct Query3 {
  float phi, z, r0, aux;  // aux: density threshold (density), rho (nearest higher)
  int li, eb, pb, self;   // self: the cluster's own position in the view
  float energy;
  bool sil;
};

// One density term (KernelCalculateDensitySoA, :26-150): candidate q of a
// row of layer cl, in the reference's operation order.
template <class V>
__device__ __forceinline__ void density_term(const V& v, const Params3D& P, const Query3& Q, float coef, int q,
                                             float& rho) {
  const float4 cj = v.rec(q);  // {roa, phi, energy, -}; q == self is the cluster itself
  const float r1 = __fmul_rn(cj.x, Q.z);
  const float dphi = reduce_range(__fsub_rn(Q.phi, cj.y), P);
  const float d0 = __fsub_rn(Q.r0, r1);
  const float a = __fmul_rn(d0, d0);
  const float c = __fmul_rn(__fmul_rn(__fmul_rn(r1, r1), dphi), dphi);
  if (__fadd_rn(a, c) < Q.aux) rho = __fadd_rn(rho, __fmul_rn((q == Q.self) ? 1.f : coef, cj.z));
}

__device__ __forceinline__ float density_coef(const Params3D& P, const Query3& Q, int cl) {
  return __fmul_rn(P.kdf, (cl == Q.li && !P.dens_same) ? 0.f : 1.f);
}

// Density terms of one row of a query's window: the clusters of the row in
// the window's phi columns, in order.
template <class V>
__device__ __forceinline__ void density_row(const V& v, const Params3D& P, const Query3& Q, const ColMask& wm, int cl,
                                            int ie, float& rho) {
  const float coef = density_coef(P, Q, cl);
  visit_row_masked(v, cl * kEtaBins + ie, wm, Q.pb - 2, Q.pb + 2,
                   [&](int q) { density_term(v, P, Q, coef, q, rho); });
}

// One cluster's nearest higher (KernelComputeDistanceToHigherSoA, :286-392)
// over the rows in `v`: best squared distance (FLT_MAX: none), its sqrt, the
// layer distance, the layer and the position in `v`.
struct Nh3 {
  float best = FLT_MAX, best_t = FLT_MAX;
  int best_l = INT_MAX, nl = -1, nq = -1;
};

template <class V>
__device__ __forceinline__ void nh_term(const V& v, const Params3D& P, const Query3& Q, int cl, int q, Nh3& o) {
  const float4 cj = v.rec(q);  // {roa, phi, energy, rho}
  const float r1 = __fmul_rn(cj.x, Q.z);
  const float dphi = reduce_range(__fsub_rn(Q.phi, cj.y), P);
  const float d0 = __fsub_rn(Q.r0, r1);
  const float d = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(__fmul_rn(__fmul_rn(r1, r1), dphi), dphi));
  if (cj.w > Q.aux && d <= o.best) {  // "<=": the last candidate wins a tie
    o.best = d;
    o.best_t = __fsqrt_rn(d);
    o.best_l = abs(cl - Q.li);
    o.nl = cl;
    o.nq = q;
  }
}

template <class V>
__device__ __forceinline__ void nh_row(const V& v, const Params3D& P, const Query3& Q, const ColMask& wm, int cl, int ie,
                                       Nh3& o) {
  visit_row_masked(v, cl * kEtaBins + ie, wm, Q.pb - 1, Q.pb + 1, [&](int q) { nh_term(v, P, Q, cl, q, o); });
}

// The window's phi columns as visited: arc A = [a0, a1] first, then arc B =
// [0, b1] when the window wraps (b1 = -1 otherwise); lt = the columns below
// a0.  All of a window's columns at or above a0 are arc A.
struct Arcs {
  unsigned long long lt0, lt1;
  int a0, a1, b1;
  __device__ __forceinline__ Arcs(int p0, int p1) {
    if (p0 < 0) {
      a0 = p0 + kPhiBins; a1 = kPhiBins - 1; b1 = p1;
    } else if (p1 >= kPhiBins) {
      a0 = p0; a1 = kPhiBins - 1; b1 = p1 - kPhiBins;
    } else {
      a0 = p0; a1 = p1; b1 = -1;
    }
    lt0 = a0 >= 64 ? ~0ull : ((1ull << a0) - 1);
    lt1 = a0 > 64 ? ((1ull << (a0 - 64)) - 1) : 0ull;
  }
};

// A live row's entries in the window, in the reference's order: the run of
// arc A, [qa, qa + na), then the run of arc B, [s, s + nb) (the row's start).
// The counts come from popcounts of the row mask plus, where a column holds
// two entries, of the repeat mask; only a row with three or more entries in
// one column is counted entry by entry (rows are short).
struct RowRuns {
  int qa, na, s, nb;
};

__device__ __forceinline__ RowRuns row_runs(const RowsStaged& v, int r, const ColMask& wm, const Arcs& ar) {
  const ulonglong2 m = v.mm(r);
  RowRuns o;
  o.s = v.start(r);
  ulonglong2 rp = make_ulonglong2(0ull, 0ull);
  if (m.y >> 63) rp = v.rep(r);
  if (!(rp.y >> 63)) {
    const unsigned long long x0 = m.x & wm.w0, x1 = m.y & wm.w1;    // columns in the window
    const unsigned long long y0 = rp.x & wm.w0, y1 = rp.y & wm.w1;  // ... holding a second entry
    o.na = __popcll(x0 & ~ar.lt0) + __popcll(x1 & ~ar.lt1) + __popcll(y0 & ~ar.lt0) + __popcll(y1 & ~ar.lt1);
    o.nb = __popcll(x0) + __popcll(x1) + __popcll(y0) + __popcll(y1) - o.na;
    o.qa = o.s + __popcll(m.x & ar.lt0) + __popcll(m.y & ar.lt1) + __popcll(rp.x & ar.lt0) + __popcll(rp.y & ar.lt1);
  } else {
    const int t = v.start(r + 1);
    int below = 0;
    o.na = o.nb = 0;
    for (int q = o.s; q < t; ++q) {
      const int c = v.col(q);
      below += c < ar.a0;
      o.na += (c >= ar.a0) & (c <= ar.a1);
      o.nb += c <= ar.b1;
    }
    o.qa = o.s + below;
  }
  return o;
}

// The window of a query: layers [lo, hi] (without `skip`), eta rows
// [e0, e1], phi columns pb +- d.
struct Window3 {
  int lo, hi, e0, e1, skip;
};

__device__ __forceinline__ Window3 window_of(const Params3D& P, const Query3& Q, bool density) {
  Window3 w;
  const int de = density ? 2 : 1;
  layer_window(Q.li, density ? P.dens_sib : P.nh_sib, P.n_layers, density ? 0 : 1, &w.lo, &w.hi);
  w.e0 = max(Q.eb - de, 0);
  w.e1 = min(Q.eb + de, kEtaBins);
  w.skip = (density || P.nh_same) ? -1 : Q.li;
  return w;
}

// A whole search over the rows of `v`, every window row in order (the rows
// whose mask shows no entry return at once).
template <bool kDensity, class V, class R>
__device__ __forceinline__ void search_all(const V& v, const Params3D& P, const Query3& Q, R& res) {
  const Window3 w = window_of(P, Q, kDensity);
  const ColMask wm(Q.pb, kDensity ? 2 : 1);
  for (int cl = w.lo; cl <= w.hi; ++cl) {
    if (cl == w.skip) continue;
    for (int ie = w.e0; ie <= w.e1; ++ie) {
      if constexpr (kDensity) density_row(v, P, Q, wm, cl, ie, res);
      else nh_row(v, P, Q, wm, cl, ie, res);
    }
  }
}

// The same search over the rows named by a live_rows() mask.
template <bool kDensity, class R>
__device__ __forceinline__ void search_live(const RowsStaged& v, const Params3D& P, const Query3& Q,
                                            unsigned long long live, R& res) {
  const Window3 w = window_of(P, Q, kDensity);
  const int d = kDensity ? 2 : 1;
  const ColMask wm(Q.pb, d);
  const Arcs ar(Q.pb - d, Q.pb + d);
  // One candidate per iteration: the lanes of a warp step through their own
  // candidate sequences together, and a lane moves to its next run (arc B of
  // the row, or the next live row) only when its current run is done.
  int q = 0, qe = 0, qb = 0, qbe = 0, cl = 0;
  float coef = 0.f;
  bool more = true;
  for (;;) {
    while (q >= qe) {
      if (qb < qbe) {
        q = qb;
        qe = qbe;
        qb = qbe = 0;
      } else if (live) {
        const int k = __ffsll((long long)live) - 1;
        live &= live - 1;
        cl = w.lo + (k >> 3);
        if constexpr (kDensity) coef = density_coef(P, Q, cl);
        const RowRuns rr = row_runs(v, cl * kEtaBins + w.e0 + (k & 7), wm, ar);
        q = rr.qa;
        qe = rr.qa + rr.na;
        qb = rr.s;
        qbe = rr.s + rr.nb;
      } else {
        more = false;
        break;
      }
    }
    if (!more) break;
    if constexpr (kDensity) density_term(v, P, Q, coef, q, res);
    else nh_term(v, P, Q, cl, q, res);
    ++q;
  }
}

// Staging of the searches: one block per (event, slab of kSlabLayers
// layers).  The block copies the rows of the slab's layers and of the
// sibling layers around them (occupancy masks, row starts, phi columns and
// the 16-byte candidate records) into shared memory once, then runs the
// searches of the slab's clusters from there (4 blocks of 256 threads per SM;
// slabs of 2, 6 and 8 layers measured slower or the same).  A cluster whose window leaves
// the staged rows (the phi bin 126 quirk can move a cluster into the next
// layer's first row) and a slab larger than the staging area read the global
// arrays instead; either way the visiting order and arithmetic are the
// reference's.
constexpr int kSlabLayers = 4;
constexpr int kSlabThreads = 256;
constexpr int kSlabMaxRows = 384;  // 10 layers of rows and one more: sibling windows up to +-3 layers
constexpr int kSlabMaxCand = 2048;
constexpr size_t kSlabSmem = 32 * (size_t)kSlabMaxRows + 4 * (size_t)(kSlabMaxRows + 1) +
                             16 * (size_t)kSlabMaxCand + (size_t)kSlabMaxCand;
static_assert(kSlabSmem <= 48 * 1024, "static shared memory");

template <bool kDensity>
__global__ void __launch_bounds__(kSlabThreads, 4) k3_search(Batch3D b, Params3D P, int n_slabs) {
  __shared__ __align__(16) unsigned char sm3[kSlabSmem];
  unsigned long long* s_mask = reinterpret_cast<unsigned long long*>(sm3);
  unsigned long long* s_rep = s_mask + 2 * kSlabMaxRows;
  float4* s_cand = reinterpret_cast<float4*>(sm3 + 32 * (size_t)kSlabMaxRows);
  int32_t* s_rs = reinterpret_cast<int32_t*>(sm3 + 32 * (size_t)kSlabMaxRows + 16 * (size_t)kSlabMaxCand);
  uint8_t* s_col = reinterpret_cast<uint8_t*>(s_rs + kSlabMaxRows + 1);
  const int e = blockIdx.x / n_slabs;
  const int L0 = (blockIdx.x % n_slabs) * kSlabLayers;
  const int L1 = min(L0 + kSlabLayers, P.n_layers);
  const int sib = kDensity ? P.dens_sib : P.nh_sib;
  const int R = b.n_rows;
  const int64_t rbase = (int64_t)e * R;
  const int32_t* rs = b.row_start + rbase;
  const int q_lo = rs[L0 * kEtaBins], q_hi = rs[L1 * kEtaBins];
  if (q_lo >= q_hi) return;
  // rows of layers [L0 - sib, L1 + sib) and the first row after them (the
  // reference's eta window reaches row 34 of a layer, the next layer's row 0)
  const int hl0 = max(L0 - max(sib, 0), 0), hl1 = min(L1 + max(sib, 0), P.n_layers);
  const int row_lo = hl0 * kEtaBins, row_hi = hl1 * kEtaBins;  // inclusive; row_hi <= R - 2
  const int nrows = row_hi - row_lo + 1;
  const int pos_lo = rs[row_lo], pos_hi = rs[row_hi + 1];
  const bool staged = nrows <= kSlabMaxRows && pos_hi - pos_lo <= kSlabMaxCand;
  if (staged) {
    const unsigned long long* gm = b.row_mask + 2 * (rbase + row_lo);
    const unsigned long long* gr = b.row_rep + 2 * (rbase + row_lo);
    for (int i = threadIdx.x; i < 2 * nrows; i += kSlabThreads) {
      s_mask[i] = gm[i];
      s_rep[i] = gr[i];
    }
    for (int i = threadIdx.x; i <= nrows; i += kSlabThreads) s_rs[i] = rs[row_lo + i] - pos_lo;
    for (int i = threadIdx.x; i < pos_hi - pos_lo; i += kSlabThreads) {
      s_cand[i] = b.cand[pos_lo + i];
      s_col[i] = (uint8_t)b.scol[pos_lo + i];
    }
    __syncthreads();
  }
  RowsStaged sv{s_mask, s_rep, s_rs, s_cand, s_col, row_lo};
  RowsGlobal gv{b.row_mask + 2 * rbase, rs, b.cand, b.scol};
  const int64_t es = b.offsets[e];
  const int tid = threadIdx.x;
  // the query rows hold only accepted clusters (rejected ones are in the
  // event's last row); a query's own data is read in sorted order
  auto query = [&](int p, bool* inside) {
    const float4 qr = b.qrec[p];
    const float4 cr = staged ? s_cand[p - pos_lo] : b.cand[p];
    const int bins = __float_as_int(qr.w);
    Query3 Q;
    Q.li = bins & 0x7ff;
    Q.eb = (bins >> 11) & 0x3f;
    Q.pb = (bins >> 17) & 0x7f;
    Q.sil = (bins >> 24) & 1;
    Q.energy = cr.z;
    Q.phi = cr.y;
    Q.z = qr.x;
    Q.r0 = qr.y;
    Q.aux = kDensity ? qr.z : cr.w;
    int lo, hi;
    layer_window(Q.li, sib, P.n_layers, kDensity ? 0 : 1, &lo, &hi);
    *inside = staged && lo * kEtaBins >= row_lo && hi * kEtaBins + kEtaBins <= row_hi;
    Q.self = *inside ? p - pos_lo : p;
    return Q;
  };
  for (int p = q_lo + tid; p < q_hi; p += kSlabThreads) {
    bool inside;
    const Query3 Q = query(p, &inside);
    const int64_t gi = es + b.sorted[p];
    // staged windows: the rows holding an entry first, in one uniform pass
    unsigned long long live = 0;
    bool by_live = false;
    if (inside) {
      const Window3 w = window_of(P, Q, kDensity);
      by_live = live_rows(sv, w.lo, w.hi, w.skip, w.e0, w.e1, ColMask(Q.pb, kDensity ? 2 : 1), &live);
    }
    if constexpr (kDensity) {
      float rho = 0.f;
      if (by_live) search_live<true>(sv, P, Q, live, rho);
      else if (inside) search_all<true>(sv, P, Q, rho);
      else search_all<true>(gv, P, Q, rho);
      b.rho[gi] = rho;
      reinterpret_cast<float*>(b.cand)[4 * (int64_t)p + 3] = rho;
    } else {
      Nh3 o;
      if (by_live) search_live<false>(sv, P, Q, live, o);
      else if (inside) search_all<false>(sv, P, Q, o);
      else search_all<false>(gv, P, Q, o);
      if (o.nq >= 0 && inside) o.nq += pos_lo;
      const bool found = o.best != FLT_MAX;
      const float dt = found ? o.best_t : FLT_MAX;
      const int dl = found ? o.best_l : INT_MAX, nl = found ? o.nl : -1;
      const int ni = found ? b.sorted[o.nq] : -1;
      b.delta_t[gi] = dt;
      b.delta_l[gi] = dl;
      b.nh_l[gi] = nl;
      b.nh_i[gi] = ni;
      // seeds and outliers (CLUE3DAlgoKernels.h:521-560); par: the nearest
      // higher for followers, -2 for seeds, -3 for other roots
      const float r = Q.aux;
      const float dxy = Q.sil ? P.crit_xy : b.radius[gi];
      const bool seed = (dt > dxy || __int2float_rn(dl) > P.crit_z) && (r >= P.crit_rho) &&
                        (__fdiv_rn(Q.energy, r) > P.crit_self);
      const bool outlier = (dt > P.out_thr) && (r < P.crit_rho);
      b.seed[gi] = seed ? 1 : 0;
      b.par[gi] = seed ? -2 : ((!outlier && nl >= 0) ? ni : -3);
    }
  }
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
  int32_t* seed = b.seed + es;
  __shared__ int s_w[16];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 512) {
    const int i = base + threadIdx.x;
    int f = (i < n) ? seed[i] : 0;
    if (f < 0) {  // rejected by k3_key: no seed, a root of its own
      f = 0;
      seed[i] = 0;
      par[i] = -3;
    }
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
  err = cudaMemsetAsync(b.row_rep, 0, 16 * (size_t)b.n_events * b.n_rows, s);
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
    k3_scatter<<<grid, T, 0, s>>>(b, p);
  }
  {
    NvtxRange r("clue3d/row_sort");
    k3_row_sort<<<grid, T, 0, s>>>(b);
  }
  const int n_slabs = (p.n_layers + kSlabLayers - 1) / kSlabLayers;
  const int64_t slab_blocks = (int64_t)b.n_events * n_slabs;
  if (slab_blocks > INT32_MAX) return cudaErrorInvalidValue;
  {
    NvtxRange r("clue3d/density");
    k3_search<true><<<(unsigned)slab_blocks, kSlabThreads, 0, s>>>(b, p, n_slabs);
  }
  {
    NvtxRange r("clue3d/nearest_higher");
    k3_search<false><<<(unsigned)slab_blocks, kSlabThreads, 0, s>>>(b, p, n_slabs);
  }
  {
    NvtxRange r("clue3d/finish");
    k3_finish<<<b.n_events, 512, 0, s>>>(b);
  }
  return cudaGetLastError();
}

}  // namespace clue
