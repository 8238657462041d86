// CLUE 2D on GB300: the four serial stages of
// src/serial/plugin-CLUEClusterizer/CLUEAlgoKernels.h re-designed for the GPU.
//
// Pipeline of one batch (events concatenated in CSR order):
//   k_init         the batch's counters, tickets and flags
//   k_count        points per (event, layer), warp-aggregated atomics; also
//                  notes whether every event is already grouped by layer
//   k_layer_scan   per-event exclusive scan -> first position of each layer
//                  (and, for batches of a few layers per CTA, layer sizes)
//   k_order        those batches only: layers in descending size
//   k_scatter      group points by (event, layer) when the input is not
//   k_layers       persistent CTAs over the (event, layer) queue (one wide
//                  pass for a single event, else one or two classes of layer
//                  size); the next layer's inputs prefetched into L2.  Per layer,
//                  on-chip: counting sort into the reference's 5 cm tiles
//                  (column-major, index order inside a tile), density,
//                  nearest-higher, seed/outlier flags (and seeds counted per
//                  event-aligned chunk of 4096 points) and pointer jumping
//                  to each point's root
//   k_seed_chunk_scan / k_seed_rank
//                  event-wide seed numbering in index order
//   k_label        clusterIndex = cluster of the root seed, -1 when the
//                  chain ends at an outlier
//
// Bit-exactness with the serial backend:
//  * candidates of a query are enumerated xBin-outer, yBin-inner, index order
//    inside a tile (CLUEAlgoKernels.h:35-44,76-85); a column-major sort key
//    makes each column's rows one contiguous range of the sorted layer;
//  * rho is a sequential float sum in that order, (i==j ? 1 : 0.5) * w_j,
//    with __fmul_rn/__fadd_rn (no contraction; the file is built --fmad=false);
//  * "sqrtf(dx*dx+dy*dy) <= d" is evaluated as "dx*dx+dy*dy <= t" with t the
//    largest float whose correctly rounded square root is <= d, which is the
//    same predicate because sqrt_rn is monotone;
//  * nearest-higher keeps the reference's strict "dist < delta" on the
//    square-rooted distance (first candidate wins a tie); the squared
//    distance only filters candidates that cannot win;
//  * seeds are numbered by rank in point-index order over the whole event
//    (CLUEAlgoKernels.h:114-131) and labels follow nearestHigher chains
//    exactly where the reference's follower stack walks (:133-152).
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

#include <algorithm>

#include "clue_internal.h"

namespace clue {

namespace {

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }

// LayerTilesSerial::getXBin / getYBin (src/serial/DataFormats/LayerTilesSerial.h:24-40):
// (v - (-250)) * 0.2 in float, truncated toward zero (saturating), clamped to
// [0, 99]; a NaN lands in bin 0 (the conversion gives 0 or INT_MIN, both
// clamped to 0), as (int)NaN does on the aarch64 host.
__device__ __forceinline__ int tile_bin(float v) {
  const int b = __float2int_rz(__fmul_rn(__fsub_rn(v, -250.f), 0.2f));
  return min(max(b, 0), kGridCols - 1);
}

// Event of a chunk: the last e with chunk_start[e] <= c (empty events own no chunk).
__device__ __forceinline__ int chunk_event(const int32_t* chunk_start, int n_events, int c) {
  int lo = 0, hi = n_events;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (chunk_start[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

// Event of a chunk: from the host-built table when the batch has one.
__device__ __forceinline__ int event_of_chunk(const Batch2D& b, int c) {
  return b.chunk_ev ? b.chunk_ev[c] : chunk_event(b.chunk_start, b.n_events, c);
}

template <int NT>
__device__ __forceinline__ int block_inclusive_scan(int v, int* s_ws, int* total) {
  constexpr int NW = NT / 32;
  const int lane = lane_id(), warp = warp_id();
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) s_ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int wv = lane < NW ? s_ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wv, o);
      if (lane >= o) wv += t;
    }
    if (lane < NW) s_ws[lane] = wv;
  }
  __syncthreads();
  const int res = x + (warp > 0 ? s_ws[warp - 1] : 0);
  *total = s_ws[NW - 1];
  __syncthreads();
  return res;
}

// Exclusive scan of tbl[0..n) in place, tbl[n] = total (32-bit counts, HBM tables).
template <int NT>
__device__ void block_scan_table(int32_t* tbl, int n, int* s_ws) {
  const int per = (n + NT - 1) / NT;
  const int beg = min((int)threadIdx.x * per, n);
  const int end = min(beg + per, n);
  int sum = 0;
  for (int i = beg; i < end; ++i) sum += tbl[i];
  int total;
  const int incl = block_inclusive_scan<NT>(sum, s_ws, &total);
  int run = incl - sum;
  for (int i = beg; i < end; ++i) {
    const int c = tbl[i];
    tbl[i] = run;
    run += c;
  }
  if (threadIdx.x == 0) tbl[n] = total;
  __syncthreads();
}

// The same for the on-chip 16-bit table: each thread scans whole 16-byte
// groups of 8 counts (kTiles = 10000 is a multiple of 8).
template <int NT>
__device__ void block_scan_table(uint16_t* tbl, int n, int* s_ws) {
  const int groups = n / 8;
  const int per = (groups + NT - 1) / NT;
  const int beg = min((int)threadIdx.x * per, groups);
  const int end = min(beg + per, groups);
  uint4* t4 = reinterpret_cast<uint4*>(tbl);
  int sum = 0;
  for (int g = beg; g < end; ++g) {
    const uint4 v = t4[g];
    const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) sum += (int)(w[j] & 0xffffu) + (int)(w[j] >> 16);
  }
  int total;
  const int incl = block_inclusive_scan<NT>(sum, s_ws, &total);
  unsigned run = (unsigned)(incl - sum);
  for (int g = beg; g < end; ++g) {
    const uint4 v = t4[g];
    unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const unsigned lo = w[j] & 0xffffu, hi = w[j] >> 16;
      w[j] = run | ((run + lo) << 16);
      run += lo + hi;
    }
    t4[g] = make_uint4(w[0], w[1], w[2], w[3]);
  }
  if (threadIdx.x == 0) tbl[n] = (uint16_t)total;
  __syncthreads();
}

// Histogram increment returning the previous count.  The on-chip table holds
// 16-bit counts (a layer there has < 65536 points), two per 32-bit word.
__device__ __forceinline__ int hist_add(uint16_t* t, int key, int n) {
  unsigned* w = reinterpret_cast<unsigned*>(t) + (key >> 1);
  const int sh = (key & 1) * 16;
  return (int)((atomicAdd(w, (unsigned)n << sh) >> sh) & 0xffffu);
}
__device__ __forceinline__ int hist_add(int32_t* t, int key, int n) { return atomicAdd(t + key, n); }

// Squared distance dx*dx + dy*dy with the reference's rounding: two
// correctly rounded differences, two correctly rounded squares (computed as
// one packed f32x2 pair each) and one correctly rounded sum.
__device__ __forceinline__ float dist2(float2 a, float2 b) {
  float sx, sy;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\t"
      "mul.rn.f32x2 pd, pd, pd;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(sx), "=f"(sy)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return __fadd_rn(sx, sy);
}

// Order-preserving map of a non-NaN float to 32 bits (rho is never -0: it
// starts at +0 and only adds terms).  NaN maps to 0, below every number.
__device__ __forceinline__ unsigned float_ord(float f) {
  const unsigned u = __float_as_uint(f);
  if (f != f) return 0u;
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_float(unsigned o) {
  if (o == 0u) return __uint_as_float(0x7fffffffu);  // NaN
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Per-layer working set, sorted by tile: on-chip for layers up to the tuned
// capacity (16-bit table and query order), in HBM scratch beyond it (32-bit).
// One 16-byte record per point, so a candidate is a single 128-bit load:
//   {x, y, gid, aux}: aux = 0.5f*w (bits) during the density search and
//   float_ord(rho) during the nearest-higher search, when the upper 8 bytes
//   read as one 64-bit key (float_ord(rho) << 32) | gid.
// 22 bytes per point on chip plus the 20 KB table.
template <class TT, class QT>
struct LayerStore {
  uint4* rec;
  int32_t* nh;  // own weight (bits), then float_ord(rho), then the parent pointer
  QT* qord;     // query order of the current search
  TT* tbl;      // kTableInts: exclusive scan over key = xBin*100 + yBin
};

struct LayerIO {
  const float* x;
  const float* y;
  const float* w;
  const int32_t* gid;  // nullptr: gid = gid_base + p
  int32_t gid_base;
  int64_t ev_start;
  int32_t chunk0;  // first seed-count chunk of the event
};

__device__ __forceinline__ float2 rec_xy(const uint4& r) { return make_float2(__uint_as_float(r.x), __uint_as_float(r.y)); }
__device__ __forceinline__ unsigned long long rec_key(const uint4& r) {
  return ((unsigned long long)r.w << 32) | r.z;
}

template <class TT>
__device__ __forceinline__ int candidate_count(const TT* tbl, int bx0, int bx1, int by0, int by1) {
  int cnt = 0;
  for (int c = bx0; c <= bx1; ++c) cnt += max(0, (int)tbl[c * kGridCols + by1 + 1] - (int)tbl[c * kGridCols + by0]);
  return cnt;
}

// Query order of a search phase: queries bucketed by their candidate count,
// heaviest first; warps then take chunks of 32 in that order, so the lanes
// of a warp run loops of similar length.  Which thread runs which query never
// changes a result.  The bucket is computed twice instead of being stored.
template <int NT, class TT, class QT>
__device__ void order_queries(const LayerStore<TT, QT>& S, const int m, const float d, int* s_bins) {
  constexpr int NB = 64;
  const int tid = threadIdx.x;
  auto bucket = [&](int q) {
    const float2 p = rec_xy(S.rec[q]);
    const int bx0 = tile_bin(__fsub_rn(p.x, d)), bx1 = tile_bin(__fadd_rn(p.x, d));
    const int by0 = tile_bin(__fsub_rn(p.y, d)), by1 = tile_bin(__fadd_rn(p.y, d));
    return NB - 1 - min(candidate_count(S.tbl, bx0, bx1, by0, by1) >> 1, NB - 1);  // 2 candidates per bucket
  };
  for (int i = tid; i < NB; i += NT) s_bins[i] = 0;
  __syncthreads();
  for (int q = tid; q < m; q += NT) atomicAdd(&s_bins[bucket(q)], 1);
  __syncthreads();
  if (tid < 32) {
    const int a = s_bins[2 * tid], c = s_bins[2 * tid + 1];
    int x = a + c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, x, o);
      if (tid >= o) x += t;
    }
    const int ex = x - a - c;
    s_bins[2 * tid] = ex;
    s_bins[2 * tid + 1] = ex + a;
  }
  __syncthreads();
  for (int q = tid; q < m; q += NT) S.qord[atomicAdd(&s_bins[bucket(q)], 1)] = (QT)q;
  __syncthreads();
}

// Candidate sequence of a search box spanning one to three tile columns:
// segment j is column bx0+j, rows [by0, by1], i.e. sorted positions
// [s_j, s_j + l_j).  at(t) maps the t-th candidate of the concatenation to
// its sorted position with compares and selects only.
struct SegIndex {
  int b1 = 0, b2 = 0, total = 0, d0 = 0, d1 = 0, d2 = 0;
  template <class TT>
  __device__ __forceinline__ void init(const TT* tbl, int bx0, int nseg, int by0, int by1) {
    int s[3] = {0, 0, 0}, l[3] = {0, 0, 0};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j < nseg) {
        const int c = (bx0 + j) * kGridCols;
        s[j] = (int)tbl[c + by0];
        l[j] = max(0, (int)tbl[c + by1 + 1] - s[j]);
      }
    }
    b1 = l[0];
    b2 = l[0] + l[1];
    total = b2 + l[2];
    d0 = s[0];
    d1 = s[1] - b1;
    d2 = s[2] - b2;
  }
  __device__ __forceinline__ int at(int t) const { return t + (t < b1 ? d0 : (t < b2 ? d1 : d2)); }
};

// Visits the candidates of a search box in the reference order: the
// branchless flattened form for boxes of up to three columns, otherwise a
// general column loop.  Both flattened loops are unrolled four times
// (4096-event batch: two-column loop unrolled 2/4/8 times 21.72/21.46/22.62
// ms, three-column loop 2/4 times 21.46/21.38 ms).
template <class TT, class F>
__device__ __forceinline__ void for_candidates(const TT* tbl, int bx0, int bx1, int by0, int by1, F&& visit) {
  const int nseg = bx1 - bx0 + 1;
  // the widest box among the active lanes picks the loop form for the warp,
  // so that lanes never split between two loops
  const unsigned act = __activemask();
  const bool any3 = __any_sync(act, nseg == 3);
  const bool anywide = __any_sync(act, nseg > 3);
  if (!any3 && !anywide) {
    // one or two columns (every density box when dc < 2.5 cm): one compare
    // and one select per candidate
    int b1 = 0, total = 0, d0 = 0, d1 = 0;
    if (nseg >= 1) {
      const int s0 = (int)tbl[bx0 * kGridCols + by0];
      const int l0 = max(0, (int)tbl[bx0 * kGridCols + by1 + 1] - s0);
      int s1 = 0, l1 = 0;
      if (nseg == 2) {
        s1 = (int)tbl[(bx0 + 1) * kGridCols + by0];
        l1 = max(0, (int)tbl[(bx0 + 1) * kGridCols + by1 + 1] - s1);
      }
      b1 = l0;
      total = l0 + l1;
      d0 = s0;
      d1 = s1 - l0;
    }
#pragma unroll 4
    for (int t = 0; t < total; ++t) visit(t + (t < b1 ? d0 : d1));
  } else if (!anywide) {
    SegIndex sg;
    sg.init(tbl, bx0, nseg, by0, by1);
#pragma unroll 4
    for (int t = 0; t < sg.total; ++t) visit(sg.at(t));
  } else {
    for (int c = bx0; c <= bx1; ++c) {
      const int e = (int)tbl[c * kGridCols + by1 + 1];
      for (int k = (int)tbl[c * kGridCols + by0]; k < e; ++k) visit(k);
    }
  }
}

// Next chunk of 32 queries for this warp (dynamic, in query order).
__device__ __forceinline__ int next_chunk(int* s_next) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(s_next, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

// One (event, layer) item through every stage.  next_item: in thread 0, the
// item this CTA takes next (-1 when none), whose inputs are prefetched.
template <int NT, class TT, class QT>
__device__ void process_layer(const Params2D& P, const LayerStore<TT, QT>& S, const int m, const LayerIO& in,
                              const Batch2D& b, int* s_ws, int* s_bins, int* s_next, int next_item) {
  const int tid = threadIdx.x, lane = tid & 31;
  QT* kkey = S.qord;                                     // sort key, later final slot
  int32_t* kprov = S.nh;                                 // provisional slot in tile
  int32_t* slot_p = reinterpret_cast<int32_t*>(S.rec);  // input position at provisional slot
  int32_t* slot_g = slot_p + m;                          // gid at provisional slot

  // -- counting sort into tiles (kernel_compute_histogram, CLUEAlgoKernels.h:18-23)
  {
    constexpr int kTableBytes = ((kTableInts * (int)sizeof(TT) + 15) / 16) * 16;
    uint4* t4 = reinterpret_cast<uint4*>(S.tbl);
    for (int i = tid; i < kTableBytes / 16; i += NT) t4[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  __syncthreads();
  {
    const unsigned lt = (1u << lane) - 1u;
    // gid = gid_base + p ascends with p (layer-ordered input); otherwise the
    // gids come from the layer-grouping gather in arbitrary order
    const bool mono = in.gid == nullptr;
    int32_t* lead_p = slot_p + 2 * m;  // by point: size of the group it leads, else 0
    int32_t* lead_q = slot_p + 3 * m;  // the same by provisional slot
    for (int base = 0; base < m; base += NT) {
      const int p = base + tid;
      const int key = p < m ? tile_bin(in.x[p]) * kGridCols + tile_bin(in.y[p]) : -1;
      const unsigned grp = __match_any_sync(0xffffffffu, key);
      const int leader = __ffs(grp) - 1;
      int old = 0;
      if (key >= 0 && lane == leader) old = hist_add(S.tbl, key, __popc(grp));
      old = __shfl_sync(0xffffffffu, old, leader);
      if (key >= 0) {
        kkey[p] = (QT)key;
        kprov[p] = old + __popc(grp & lt);
        if (mono) lead_p[p] = lane == leader ? __popc(grp) : 0;
      }
    }
    __syncthreads();
    block_scan_table<NT>(S.tbl, kTiles, s_ws);
    for (int p = tid; p < m; p += NT) {
      const int q = (int)S.tbl[kkey[p]] + kprov[p];
      slot_g[q] = in.gid ? in.gid[p] : in.gid_base + p;
      slot_p[q] = p;
      if (mono) lead_q[q] = lead_p[p];
    }
    __syncthreads();
    // Atomics gave an arbitrary order inside a tile; the reference appends in
    // index order, so place each point at its gid rank within the tile.  With
    // layer-ordered input a tile's slots are groups (one atomic each) of lanes
    // of one warp pass over 32 consecutive points: gids ascend inside a group
    // and different groups cover disjoint gid ranges, so the rank is the sizes
    // of the groups that start below g plus g's place in its own group -- a
    // walk over the tile's groups instead of its points.
    for (int q = tid; q < m; q += NT) {
      const int p = slot_p[q];
      const int key = (int)kkey[p];
      const int s = (int)S.tbl[key], e = (int)S.tbl[key + 1];
      const int g = slot_g[q];
      int rank = 0;
      if (mono) {
        for (int t = s; t < e;) {
          const int c = max(lead_q[t], 1);
          if (q >= t && q < t + c) rank += q - t;
          else if (slot_g[t] < g) rank += c;
          t += c;
        }
      } else {
        for (int t = s; t < e; ++t) rank += (slot_g[t] < g);
      }
      kkey[p] = (QT)(s + rank);
    }
    __syncthreads();
  }
  for (int p = tid; p < m; p += NT) {
    const int f = (int)kkey[p];
    const float wv = in.w[p];
    const unsigned g = (unsigned)(in.gid ? in.gid[p] : in.gid_base + p);
    S.rec[f] = make_uint4(__float_as_uint(in.x[p]), __float_as_uint(in.y[p]), g, __float_as_uint(__fmul_rn(0.5f, wv)));
    S.nh[f] = __float_as_int(wv);
  }
  __syncthreads();

  // the next layer's inputs (the ticket taken while this layer started) into
  // L2 while this one is searched: its histogram and records then read L2
  if (tid < 32) {
    const int nx = __shfl_sync(0xffffffffu, next_item, 0);
    if (nx >= 0) {
      const int nm = b.lcnt[nx];
      const int ns = b.lstart[nx];
      const bool gr = b.flags[kFlagGrouped] != 0;
      const float* ax = (gr ? b.x : b.gx) + ns;
      const float* ay = (gr ? b.y : b.gy) + ns;
      const float* aw = (gr ? b.w : b.gw) + ns;
      for (int o = lane * 32; o < nm; o += 32 * 32) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(ax + o));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(ay + o));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(aw + o));
      }
    }
  }

  // One query order for both searches, by the nearest-higher box (the
  // larger box and the more expensive search).  Layers of up to 256 points
  // keep the input order: there the ordering costs more than it saves
  // (4096-event batch: k_layers 21.58 -> 21.46 ms; 21.59 ms with the
  // threshold at 512).
  if (m > 256) {
    order_queries<NT>(S, m, P.dm, s_bins);
  } else {
    for (int i = tid; i < m; i += NT) S.qord[i] = (QT)i;
    __syncthreads();
  }

  // -- local density (kernel_calculate_density, CLUEAlgoKernels.h:25-55)
  if (tid == 0) *s_next = 0;
  __syncthreads();
  for (;;) {
    const int base = next_chunk(s_next);
    if (base >= m) break;
    const int i = base + lane;
    if (i < m) {
      const int q = (int)S.qord[i];
      const uint4 rq = S.rec[q];
      const float2 pq = rec_xy(rq);
      const float wq = __int_as_float(S.nh[q]);
      const int bx0 = tile_bin(__fsub_rn(pq.x, P.dc)), bx1 = tile_bin(__fadd_rn(pq.x, P.dc));
      const int by0 = tile_bin(__fsub_rn(pq.y, P.dc)), by1 = tile_bin(__fadd_rn(pq.y, P.dc));
      float r = 0.f;
      for_candidates(S.tbl, bx0, bx1, by0, by1, [&](int k) {
        const uint4 rk = S.rec[k];
        const float h = (k == q) ? wq : __uint_as_float(rk.w);  // the i == j term is w, not 0.5 w
        if (dist2(pq, rec_xy(rk)) <= P.t_dc) r = __fadd_rn(r, h);
      });
      b.rho[in.ev_start + rq.z] = r;
      S.nh[q] = (int)float_ord(r);  // nobody reads nh[q] during this search but this thread
    }
  }
  __syncthreads();
  for (int q = tid; q < m; q += NT) S.rec[q].w = (unsigned)S.nh[q];
  __syncthreads();

  // -- distance to the nearest higher (kernel_calculate_distanceToHigher, :57-106)
  // "higher" (rho_j > rho_i, or equal rho and j > i) is key_j > key_i; a NaN
  // rho is higher than nothing and nothing is higher than it, as in the
  // reference.  The winner is the first candidate with the smallest
  // correctly rounded sqrt(d2).  The loop keeps the first candidate with the
  // smallest d2 and takes the exact sqrt comparison only for near ties:
  //   d2 < 0.99999 * best_d2  implies  sqrt_rn(d2) < sqrt_rn(best_d2),
  // so a candidate below `lim` always wins, one at or above best_d2 never
  // does (sqrt_rn is monotone), and one in between is decided by sqrt_rn.
  if (tid == 0) *s_next = 0;
  __syncthreads();
  int32_t* par = S.nh;  // parent: nearest higher for followers, -2 seed root, -3 other root
  for (;;) {
    const int base = next_chunk(s_next);
    if (base >= m) break;
    const int i = base + lane;
    if (i < m) {
      const int q = (int)S.qord[i];
      const uint4 rq = S.rec[q];
      const float2 pq = rec_xy(rq);
      const unsigned long long ks = rec_key(rq);
      const unsigned long long kq = rq.w == 0u ? ~0ull : ks;
      const int bx0 = tile_bin(__fsub_rn(pq.x, P.dm)), bx1 = tile_bin(__fadd_rn(pq.x, P.dm));
      const int by0 = tile_bin(__fsub_rn(pq.y, P.dm)), by1 = tile_bin(__fadd_rn(pq.y, P.dm));
      float best_d2 = P.t_dm_next;  // d2 < t_dm_next <=> d2 <= t_dm
      int best = -1;
      bool near = false;
      for_candidates(S.tbl, bx0, bx1, by0, by1, [&](int k) {
        const uint4 rk = S.rec[k];
        const float d2 = dist2(pq, rec_xy(rk));
        const bool imp = (rec_key(rk) > kq) && d2 < best_d2;
        // d2 * 1.00002 < best_d2 guarantees sqrt_rn(d2) < sqrt_rn(best_d2)
        const bool win = imp && __fmul_rn(d2, 1.00002f) < best_d2;
        near |= imp && !win;
        best = win ? k : best;
        best_d2 = win ? d2 : best_d2;
      });
      float best_s = best >= 0 ? __fsqrt_rn(best_d2) : FLT_MAX;
      if (near) {
        // a candidate came within the margin of the running best: decide this
        // query again with the reference's comparison on sqrt'd distances
        best_s = FLT_MAX;
        best = -1;
        for_candidates(S.tbl, bx0, bx1, by0, by1, [&](int k) {
          const uint4 rk = S.rec[k];
          const float d2 = dist2(pq, rec_xy(rk));
          if (rec_key(rk) > kq && d2 <= P.t_dm) {
            const float sd = __fsqrt_rn(d2);
            if (sd < best_s) {
              best_s = sd;
              best = k;
            }
          }
        });
      }
      // -- seeds, outliers, outputs (kernel_findAndAssign_clusters, :108-136)
      const float r = ord_float(rq.w);
      const bool seed = (best_s > P.dc) && (r >= P.rhoc);
      const bool outlier = (best_s > P.dm) && (r < P.rhoc);
      const int64_t o = in.ev_start + rq.z;
      b.delta[o] = best_s;
      b.nh[o] = best >= 0 ? (int)S.rec[best].z : -1;
      b.seed[o] = seed ? 1 : 0;
      // seeds per event-aligned chunk of 4096 points, for the seed ranks
      if (seed) atomicAdd(&b.chunk_seeds[in.chunk0 + (int)(rq.z / kChunk)], 1);
      par[q] = (!seed && !outlier && best >= 0) ? best : (seed ? -2 : -3);
    }
  }
  __syncthreads();
  // -- roots of the nearestHigher chains (replaces the follower stack,
  // :138-152): each point walks its chain; chains longer than 64 steps are
  // finished by pointer jumping.
  QT* root = S.qord;  // the query order is not needed any more
  int unresolved = 0;
  for (int q = tid; q < m; q += NT) {
    int r = q, p = par[q];
    for (int step = 0; p >= 0 && step < 64; ++step) {
      r = p;
      p = par[r];
    }
    root[q] = (QT)r;
    unresolved |= (p >= 0);
  }
  if (__syncthreads_or(unresolved)) {
    for (;;) {
      int changed = 0;
      for (int q = tid; q < m; q += NT) {
        const int p = par[q];
        if (p >= 0) {
          const int pp = par[p];
          if (pp >= 0) {
            par[q] = pp;
            changed = 1;
          }
        }
      }
      if (!__syncthreads_or(changed)) break;
    }
    for (int q = tid; q < m; q += NT) root[q] = (QT)(par[q] >= 0 ? par[q] : q);
    __syncthreads();
  }
  for (int q = tid; q < m; q += NT) {
    const int r = (int)root[q];
    // a chain ending at a seed carries -(seed's event-local index + 2) until
    // k_seed_rank (seeds) and k_label (the others) put the seed's rank there
    b.ci[in.ev_start + S.rec[q].z] = (par[r] == -2) ? -((int)S.rec[r].z + 2) : -1;
  }
  __syncthreads();
}
// ------------------------------------------------------------------ kernels

// Per-batch counters to their start values: layer counts and per-chunk seed
// counts to 0, the tickets and pass counters to 0, "grouped" to 1 (k_count
// clears it on the first layer decrease).  The error word is left alone: it
// accumulates over the launches of a run.
__global__ void k_init(Batch2D b, int64_t n_lcnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n_lcnt) b.lcnt[i] = 0;
  if (i < b.n_chunks) b.chunk_seeds[i] = 0;
  if (i < kFlagCount - kFlagTicket) b.flags[kFlagTicket + i] = 0;
  if (i == 0) b.flags[kFlagGrouped] = 1;
}

__global__ void __launch_bounds__(kChunkThreads) k_count(Batch2D b) {
  const int c = blockIdx.x;
  __shared__ int s_e;
  __shared__ int s_cnt[kLayers];
  for (int l = threadIdx.x; l < kLayers; l += kChunkThreads) s_cnt[l] = 0;
  // the size histogram of k_layer_scan starts from zero (it runs after this kernel)
  if (c == 0 && b.use_order)
    for (int i = threadIdx.x; i < 2 * kSizeBuckets; i += kChunkThreads) b.size_hist[i] = 0;
  if (threadIdx.x == 0) s_e = event_of_chunk(b, c);
  __syncthreads();
  const int e = s_e;
  const int64_t es = b.offsets[e], ee = b.offsets[e + 1];
  const int64_t i0 = es + (int64_t)(c - b.chunk_start[e]) * kChunk;
  const int64_t i1 = min(i0 + (int64_t)kChunk, ee);
  const int lane = lane_id();
  bool ungrouped = false;
  // all loads of the chunk first, so that they are in flight together
  constexpr int PER = kChunk / kChunkThreads;
  int lv[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t i = i0 + threadIdx.x + (int64_t)j * kChunkThreads;
    lv[j] = i < i1 ? b.layer[i] : 0;
  }
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t i = i0 + threadIdx.x + (int64_t)j * kChunkThreads;
    int key = -1;
    const int l = lv[j];
    if (i < i1) {
      if (l < 0 || l >= kLayers) {
        atomicExch(&b.flags[kFlagError], 1);
        ungrouped = true;
      } else {
        key = l;
      }
    }
    // grouped input: a point's layer is not below its predecessor's (the
    // predecessor of lane 0 is read from memory, the others by shuffle)
    const int prev = __shfl_up_sync(0xffffffffu, l, 1);
    if (key >= 0 && i > es) {
      const int pl = lane ? prev : b.layer[i - 1];
      if (l < pl) ungrouped = true;
    }
    // most warps of grouped input hold one layer: one increment for the warp
    const int k0 = __shfl_sync(0xffffffffu, key, 0);
    if (__all_sync(0xffffffffu, key == k0)) {
      if (lane == 0 && k0 >= 0) atomicAdd(&s_cnt[k0], 32);
    } else {
      const unsigned mask = __match_any_sync(0xffffffffu, key);
      if (key >= 0 && lane == __ffs(mask) - 1) atomicAdd(&s_cnt[key], __popc(mask));
    }
  }
  if (__syncthreads_or(ungrouped) && threadIdx.x == 0) b.flags[kFlagGrouped] = 0;
  for (int l = threadIdx.x; l < kLayers; l += kChunkThreads)
    if (s_cnt[l]) atomicAdd(&b.lcnt[e * kLayers + l], s_cnt[l]);
}

// Size class of a non-empty layer: 0 for the largest.
__device__ __forceinline__ int size_bucket(int m) { return kSizeBuckets - 1 - min(m >> 4, kSizeBuckets - 1); }

// One warp per event: layers 4*lane .. 4*lane+3.  Also counts the non-empty
// layers per size class for k_order.
__global__ void k_layer_scan(Batch2D b) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= b.n_events) return;
  const int lane = lane_id();
  int c[4];
  int sum = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int l = lane * 4 + j;
    c[j] = l < kLayers ? b.lcnt[e * kLayers + l] : 0;
    sum += c[j];
  }
  int x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  int run = (int)b.offsets[e] + x - sum;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int l = lane * 4 + j;
    if (l < kLayers) {
      b.lstart[e * kLayers + l] = run;
      b.cursor[e * kLayers + l] = run;
    }
    run += c[j];
    if (!b.use_order) continue;
    const int key = c[j] > 0 ? size_bucket(c[j]) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(grp) - 1) atomicAdd(&b.size_hist[key], __popc(grp));
  }
}

// The non-empty (event, layer) items in descending size class (a counting
// sort over the classes; the order inside a class is arbitrary).  The layer
// kernel takes its tickets in this order, so each pass ends on its smallest
// layers instead of on whichever layer came last.  Which CTA runs which
// layer never changes a result.  One warp per event; 256 threads per block,
// one per size class for the scan.
__global__ void __launch_bounds__(kSizeBuckets) k_order(Batch2D b) {
  static_assert(kSizeBuckets == 256, "one thread per size class");
  __shared__ int s_base[kSizeBuckets];
  __shared__ int s_ws[33];
  const int tid = threadIdx.x;
  const int v = b.size_hist[tid];
  int total;
  const int inc = block_inclusive_scan<kSizeBuckets>(v, s_ws, &total);
  s_base[tid] = inc - v;
  if (blockIdx.x == 0 && tid == 0) b.flags[kFlagOrdered] = total;
  __syncthreads();
  const int e = (blockIdx.x * blockDim.x + tid) >> 5;
  if (e >= b.n_events) return;
  const int lane = lane_id();
  const unsigned lt = (1u << lane) - 1u;
  for (int l0 = 0; l0 < kLayers; l0 += 32) {
    const int l = l0 + lane;
    const int m = l < kLayers ? b.lcnt[e * kLayers + l] : 0;
    const int key = m > 0 ? size_bucket(m) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(grp) - 1;
    int pos = 0;
    if (key >= 0 && lane == leader) pos = atomicAdd(&b.size_hist[kSizeBuckets + key], __popc(grp));
    pos = __shfl_sync(0xffffffffu, pos, leader);
    if (key >= 0) b.order[s_base[key] + pos + __popc(grp & lt)] = e * kLayers + l;
  }
}

__global__ void __launch_bounds__(kChunkThreads) k_scatter(Batch2D b) {
  if (b.flags[kFlagGrouped]) return;  // input already grouped by layer
  const int c = blockIdx.x;
  __shared__ int s_e;
  if (threadIdx.x == 0) s_e = event_of_chunk(b, c);
  __syncthreads();
  const int e = s_e;
  const int64_t es = b.offsets[e], ee = b.offsets[e + 1];
  const int64_t i0 = es + (int64_t)(c - b.chunk_start[e]) * kChunk;
  const int64_t i1 = min(i0 + (int64_t)kChunk, ee);
  const unsigned lt = (1u << lane_id()) - 1u;
  for (int64_t base = i0; base < i1; base += kChunkThreads) {
    const int64_t i = base + threadIdx.x;
    int key = -1;
    if (i < i1) {
      const int l = b.layer[i];
      if (l >= 0 && l < kLayers) key = e * kLayers + l;
    }
    const unsigned mask = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(mask) - 1;
    int pos = 0;
    if (key >= 0 && lane_id() == leader) pos = atomicAdd(&b.cursor[key], __popc(mask));
    pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(mask & lt);
    if (key >= 0) {
      b.gx[pos] = b.x[i];
      b.gy[pos] = b.y[i];
      b.gw[pos] = b.w[i];
      b.gid[pos] = (int32_t)(i - es);
    }
  }
}

// Persistent CTAs over the (event, layer) queue, in event order or, when
// launched with use_order, largest layers first (k_order).  Two classes of layers: the
// first pass (big_pass = 0) takes every item from an atomic ticket and
// handles layers of at most max_m points on chip with `cap` points of shared
// memory (several CTAs per SM); larger layers are appended to a list that the
// second pass (big_pass = 1, launched with a large `cap` and fewer CTAs per
// SM) drains.  Layers above `cap` in either pass use HBM scratch.
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_layers(Batch2D b, Params2D P, int cap, int max_m, int big_pass) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ int s_item;
  __shared__ int s_next;
  __shared__ int s_ws[33];
  __shared__ int s_bins[64];
  const int n_items = b.use_order ? b.flags[kFlagOrdered] : b.n_events * kLayers;
  const bool grouped = b.flags[kFlagGrouped] != 0;
  LayerStore<uint16_t, uint16_t> sm;
  sm.tbl = reinterpret_cast<uint16_t*>(dsm);
  sm.rec = reinterpret_cast<uint4*>(dsm + kSmemTableBytes);
  sm.nh = reinterpret_cast<int32_t*>(sm.rec + cap);
  sm.qord = reinterpret_cast<uint16_t*>(sm.nh + cap);
  int32_t* big_list = b.cursor;  // k_scatter's cursors are dead by now
  // The next ticket is taken as soon as the current item is known and only
  // published at the next iteration, so the atomic's round trip overlaps the
  // current layer instead of holding the whole CTA at a barrier.
  auto fetch = [&]() {
    if (!big_pass) {
      const int t = atomicAdd(&b.flags[kFlagTicket], 1);
      if (t >= n_items) return -1;
      return b.use_order ? b.order[t] : t;
    }
    const int t = atomicAdd(&b.flags[kFlagTicket2], 1);
    return t < b.flags[kFlagBigCount] ? big_list[t] : -1;
  };
  int next = threadIdx.x == 0 ? fetch() : -1;
  for (;;) {
    if (threadIdx.x == 0) s_item = next;
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item < 0) break;
    if (threadIdx.x == 0) next = fetch();
    const int m = b.lcnt[item];
    if (m == 0) continue;
    if (m > max_m) {  // first pass: leave it to the large-capacity pass
      if (threadIdx.x == 0) big_list[atomicAdd(&b.flags[kFlagBigCount], 1)] = item;
      continue;
    }
    const int e = item / kLayers;
    const int64_t es = b.offsets[e];
    const int start = b.lstart[item];
    LayerIO io;
    io.ev_start = es;
    io.chunk0 = b.chunk_start[e];
    if (grouped) {
      io.x = b.x + start;
      io.y = b.y + start;
      io.w = b.w + start;
      io.gid = nullptr;
      io.gid_base = (int32_t)(start - es);
    } else {
      io.x = b.gx + start;
      io.y = b.gy + start;
      io.w = b.gw + start;
      io.gid = b.gid + start;
      io.gid_base = 0;
    }
    if (m <= cap) {
      process_layer<NT>(P, sm, m, io, b, s_ws, s_bins, &s_next, next);
    } else {
      // spill: the same stages on HBM scratch at this layer's grouped position
      LayerStore<int32_t, int32_t> g;
      g.rec = reinterpret_cast<uint4*>(b.sp[0]) + start;
      g.nh = reinterpret_cast<int32_t*>(b.sp[4]) + start;
      g.qord = reinterpret_cast<int32_t*>(b.sp[5]) + start;
      g.tbl = b.sp_tbl + (size_t)blockIdx.x * kTableStride;
      if (threadIdx.x == 0) atomicAdd(&b.flags[kFlagSpilled], 1);
      process_layer<NT>(P, g, m, io, b, s_ws, s_bins, &s_next, next);
    }
  }
}
// One warp per event: exclusive scan of its chunks' seed counts.
__global__ void k_seed_chunk_scan(Batch2D b) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= b.n_events) return;
  const int lane = lane_id();
  const int c0 = b.chunk_start[e], c1 = b.chunk_start[e + 1];
  int run = 0;
  for (int base = c0; base < c1; base += 32) {
    const int c = base + lane;
    const int v = c < c1 ? b.chunk_seeds[c] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (c < c1) b.chunk_base[c] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
}

// Cluster id of each seed = its rank among the event's seeds in index order.
__global__ void __launch_bounds__(kChunkThreads) k_seed_rank(Batch2D b) {
  constexpr int PER = kChunk / kChunkThreads;
  const int c = blockIdx.x;
  __shared__ int s_e;
  __shared__ int s_ws[33];
  if (threadIdx.x == 0) s_e = event_of_chunk(b, c);
  __syncthreads();
  const int e = s_e;
  const int64_t es = b.offsets[e], ee = b.offsets[e + 1];
  const int64_t i0 = es + (int64_t)(c - b.chunk_start[e]) * kChunk;
  const int64_t i1 = min(i0 + (int64_t)kChunk, ee);
  const int64_t my0 = i0 + (int64_t)threadIdx.x * PER;
  int f[PER];
  int sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    f[j] = (my0 + j < i1) ? b.seed[my0 + j] : 0;
    sum += f[j];
  }
  int total;
  const int incl = block_inclusive_scan<kChunkThreads>(sum, s_ws, &total);
  int run = b.chunk_base[c] + incl - sum;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    if (f[j]) b.ci[my0 + j] = run;
    run += f[j];
  }
}

__global__ void __launch_bounds__(kChunkThreads) k_label(Batch2D b) {
  const int c = blockIdx.x;
  __shared__ int s_e;
  if (threadIdx.x == 0) s_e = event_of_chunk(b, c);
  __syncthreads();
  const int e = s_e;
  const int64_t es = b.offsets[e], ee = b.offsets[e + 1];
  const int64_t i0 = es + (int64_t)(c - b.chunk_start[e]) * kChunk;
  const int64_t i1 = min(i0 + (int64_t)kChunk, ee);
  const int64_t n_ev = ee - es;
  // ci holds a seed's rank (>= 0, from k_seed_rank), -1 (no cluster), or
  // -(root + 2) for a point whose chain ends at the seed `root` (event-local
  // index); only the last kind is rewritten, with the root's rank.  Points
  // with an invalid layer were never written, so the root is range-checked.
  // The roots are seeds, which this kernel never writes; the gathers of one
  // thread's points are issued together.
  constexpr int PER = kChunk / kChunkThreads;
  int v[PER], r[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t i = i0 + threadIdx.x + (int64_t)j * kChunkThreads;
    v[j] = i < i1 ? b.ci[i] : -1;
  }
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t root = -(int64_t)v[j] - 2;
    r[j] = (v[j] <= -2 && root < n_ev) ? b.ci[es + root] : -1;
  }
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t i = i0 + threadIdx.x + (int64_t)j * kChunkThreads;
    if (i < i1 && v[j] <= -2) b.ci[i] = r[j];
  }
}

template <int NT>
cudaError_t launch_layers(const Batch2D& b, const Params2D& p, int cap, int max_m, int big_pass, int grid,
                          cudaStream_t s) {
  Tuning2D t;
  t.layer_capacity = cap;
  k_layers<NT><<<grid, NT, layer_smem_bytes(t), s>>>(b, p, cap, max_m, big_pass);
  return cudaGetLastError();
}

cudaError_t launch_layers_any(int threads, const Batch2D& b, const Params2D& p, int cap, int max_m, int big_pass,
                              int grid, cudaStream_t s) {
  switch (threads) {
    case 128: return launch_layers<128>(b, p, cap, max_m, big_pass, grid, s);
    case 256: return launch_layers<256>(b, p, cap, max_m, big_pass, grid, s);
    case 1024: return launch_layers<1024>(b, p, cap, max_m, big_pass, grid, s);
    default: return launch_layers<512>(b, p, cap, max_m, big_pass, grid, s);
  }
}

template <int NT>
cudaError_t allow_max_smem(int optin) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_layers<NT>);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_layers<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)a.sharedSizeBytes);
}

}  // namespace

cudaError_t prepare_clue2d_kernels(int device) {
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e != cudaSuccess) return e;
  if ((e = allow_max_smem<128>(optin)) != cudaSuccess) return e;
  if ((e = allow_max_smem<256>(optin)) != cudaSuccess) return e;
  if ((e = allow_max_smem<512>(optin)) != cudaSuccess) return e;
  if ((e = allow_max_smem<1024>(optin)) != cudaSuccess) return e;
  // Asking for a kernel's attributes loads its code on this device (the
  // runtime loads kernels lazily, at first use, by default), so that no
  // later launch of the pipeline has code to load.
  const void* rest[] = {reinterpret_cast<const void*>(k_init), reinterpret_cast<const void*>(k_count),
                        reinterpret_cast<const void*>(k_layer_scan), reinterpret_cast<const void*>(k_order),
                        reinterpret_cast<const void*>(k_scatter), reinterpret_cast<const void*>(k_seed_chunk_scan),
                        reinterpret_cast<const void*>(k_seed_rank), reinterpret_cast<const void*>(k_label)};
  for (const void* f : rest) {
    cudaFuncAttributes a;
    if ((e = cudaFuncGetAttributes(&a, f)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

float sqrt_le_threshold(float d) {
  // P(t) = sqrtf(t) <= d is monotone over t >= 0; binary search over the
  // ordered bit patterns of non-negative finite floats.
  if (!(sqrtf(0.f) <= d)) return -1.f;
  uint32_t lo = 0, hi = 0x7f7fffffu;  // P(lo) holds
  auto val = [](uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  if (sqrtf(val(hi)) <= d) return val(hi);
  while (hi - lo > 1) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (sqrtf(val(mid)) <= d) lo = mid; else hi = mid;
  }
  return val(lo);
}

Params2D make_params2d(float dc, float rhoc, float odf) {
  Params2D p;
  p.dc = dc;
  p.rhoc = rhoc;
  p.odf = odf;
  volatile float a = odf, c = dc;
  p.dm = a * c;
  p.t_dc = sqrt_le_threshold(dc);
  p.t_dm = sqrt_le_threshold(p.dm);
  // the next float above t_dm (d2 < t_dm_next <=> d2 <= t_dm); -1 stays -1
  p.t_dm_next = p.t_dm < 0.f ? p.t_dm : nextafterf(p.t_dm, INFINITY);
  return p;
}

size_t layer_smem_bytes(const Tuning2D& t) {
  // 16-bit tile table, then 22 bytes per point (see LayerStore)
  return (size_t)kSmemTableBytes + (size_t)t.layer_capacity * 22;
}

int layer_grid_max(const Tuning2D& t, int n_items) {
  int g = layer_grid(t, n_items);
  if (t.big_threads > 0 && t.big_capacity > t.layer_capacity) {
    Tuning2D big;
    big.threads = t.big_threads;
    big.layer_capacity = t.big_capacity;
    const int g2 = layer_grid(big, n_items);
    g = g2 > g ? g2 : g;
  }
  return g;
}

int layer_grid(const Tuning2D& t, int n_items) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int per_sm = t.ctas_per_sm;
  if (per_sm <= 0) {
    // resident CTAs per SM as the hardware sees them (registers, shared memory, threads)
    const size_t smem = layer_smem_bytes(t);
    cudaError_t e = cudaErrorInvalidValue;
    switch (t.threads) {
      case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_layers<128>, 128, smem); break;
      case 256: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_layers<256>, 256, smem); break;
      case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_layers<512>, 512, smem); break;
      case 1024: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_layers<1024>, 1024, smem); break;
      default: break;
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm = per_sm < 1 ? 1 : per_sm;
  }
  int g = sms * per_sm;
  if (g > n_items) g = n_items;  // never more CTAs than (event, layer) items: see launch_clue2d
  return g < 1 ? 1 : g;
}

cudaError_t launch_clue2d(const Batch2D& batch, const Params2D& p, const Tuning2D& t, cudaStream_t s,
                          cudaEvent_t* ev, int64_t* kernels) {
  if (batch.n_events <= 0 || batch.n_points <= 0) return cudaSuccess;
  // Largest layers first only where a pass ends on a visible tail: a few
  // layers per CTA (a sub-batch, a served batch).  With one layer per CTA or
  // less (a single event) every layer starts at once, and with hundreds per
  // CTA the tail is negligible and the event order measured faster.
  Batch2D b = batch;
  {
    const int n_items = b.n_events * kLayers;
    const int g = layer_grid(t, n_items);
    b.use_order = (n_items > g && n_items <= 64 * g) ? 1 : 0;
  }
  cudaError_t err;
  auto mark = [&](int i) {
    if (ev) cudaEventRecord(ev[i], s);
  };
  const int nc = b.n_chunks;
  {
    // counters, tickets and flags of this batch (seeds per chunk are counted
    // by k_layers as it flags them)
    const int64_t n_lcnt = (int64_t)b.n_events * kLayers;
    const int64_t n_init = std::max<int64_t>(std::max<int64_t>(n_lcnt, nc), kFlagCount);
    NvtxRange r("clue2d/init");
    k_init<<<(unsigned)((n_init + 255) / 256), 256, 0, s>>>(b, n_lcnt);
  }
  const int warps_grid = (b.n_events * 32 + 255) / 256;
  mark(0);
  {
    NvtxRange r("clue2d/count");
    k_count<<<nc, kChunkThreads, 0, s>>>(b);
  }
  mark(1);
  {
    NvtxRange r("clue2d/layer_scan");
    k_layer_scan<<<warps_grid, 256, 0, s>>>(b);
    if (b.use_order) k_order<<<warps_grid, kSizeBuckets, 0, s>>>(b);
  }
  mark(2);
  {
    NvtxRange r("clue2d/scatter");
    k_scatter<<<nc, kChunkThreads, 0, s>>>(b);
  }
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  mark(3);
  const int n_items = b.n_events * kLayers;
  // No more layers than SMs (a single event): one pass of the widest CTA per
  // layer, so that each layer's phases spread over 32 warps and large layers
  // stay on chip.  Measured per producer call: 0.177 -> 0.131 ms on events of
  // 150k-200k points, 0.136 -> 0.117 ms on 50k-150k, 0.113 -> 0.101 ms on 5k-20k.
  Tuning2D tt = t;
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (n_items <= sms) {
      tt.threads = 1024;
      tt.layer_capacity = std::max(std::max(t.layer_capacity, t.big_capacity), 4096);
      tt.ctas_per_sm = 0;
      tt.big_threads = tt.big_capacity = 0;
    }
  }
  const bool two_class = tt.big_threads > 0 && tt.big_capacity > tt.layer_capacity;
  // Invariant: every layer-kernel grid is at most n_items = n_events * kLayers
  // (layer_grid caps it there).  The per-CTA HBM tile tables of the spill
  // path are sized on it: one table per (event, layer) at most, e.g. 100 for
  // a single event, which the allocation-free entry point relies on.
  {
    NvtxRange r("clue2d/layers");
    err = launch_layers_any(tt.threads, b, p, tt.layer_capacity, two_class ? tt.layer_capacity : INT_MAX, 0,
                            layer_grid(tt, n_items), s);
    if (err == cudaSuccess && two_class) {
      Tuning2D big;
      big.threads = tt.big_threads;
      big.layer_capacity = tt.big_capacity;
      err = launch_layers_any(tt.big_threads, b, p, tt.big_capacity, INT_MAX, 1, layer_grid(big, n_items), s);
    }
  }
  if (err != cudaSuccess) return err;
  mark(4);
  {
    NvtxRange r("clue2d/seed_chunk_scan");
    k_seed_chunk_scan<<<warps_grid, 256, 0, s>>>(b);
  }
  mark(5);
  {
    NvtxRange r("clue2d/seed_rank");
    k_seed_rank<<<nc, kChunkThreads, 0, s>>>(b);
  }
  mark(6);
  {
    NvtxRange r("clue2d/label");
    k_label<<<nc, kChunkThreads, 0, s>>>(b);
  }
  mark(7);
  if (kernels) *kernels += 8 + (b.use_order ? 1 : 0) + (two_class ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace clue

namespace clue {
namespace {

// Order-sensitive 64-bit digest of a word array: sum of w[i] * (2i+1) * K.
__global__ void k_digest(const uint32_t* a, int64_t n, unsigned long long* out) {
  unsigned long long acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (unsigned long long)a[i] * (2ull * (unsigned long long)i + 1ull) * 0x9E3779B97F4A7C15ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

}  // namespace

cudaError_t launch_digest(const void* words, int64_t n_words, unsigned long long* d_out, cudaStream_t s) {
  if (n_words <= 0) return cudaSuccess;
  int blocks = (int)((n_words + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_digest<<<blocks, 256, 0, s>>>(static_cast<const uint32_t*>(words), n_words, d_out);
  return cudaGetLastError();
}

}  // namespace clue
