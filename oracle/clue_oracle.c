/*
 * Test infrastructure, not product code.
 *
 * CPU restatement of the serial CLUE algorithms of tonydp03/heterogeneous-clue.
 * It is the oracle: tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py call it to check (and time beside) the CUDA path.  The product
 * library never links it.
 *
 * Pinned against the unmodified reference: tests/test_oracle.py runs both on
 * seeded inputs (when the reference tree is present) and against the golden
 * vectors in tests/golden/, which tests/golden/make_golden.py wrote by running
 * the reference itself.
 *
 * Compile with -O2 -ffp-contract=off: contracting a*b+c into an FMA changes
 * delta bits, and the reference's own build leaves that to the host compiler.
 *
 * Two deliberate definitions where the reference has undefined behaviour:
 *  - float -> int bin conversion saturates (INT_MAX/INT_MIN, NaN -> 0), as
 *    aarch64 and CUDA's cvt.rzi do; x86 gives INT_MIN for huge values.
 *  - CLUE3D tiles are one flat array over layers, as the reference's
 *    std::array<std::array<std::vector>>> lays them out in memory, so an
 *    eta row index of 34 lands in the next layer's row 0 exactly as there.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* CLUE 2D                                                                    */
/* ------------------------------------------------------------------------- */

/* src/serial/DataFormats/LayerTilesConstants.h:7-26 */
#define O2_NLAYERS 100
#define O2_NCOLS 100
#define O2_NROWS 100
#define O2_NTILES (O2_NCOLS * O2_NROWS)

static int sat_f2i(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT_MAX;
  if (v < -2147483648.0f) return INT_MIN;
  return (int)v;
}

/* LayerTilesSerial::getXBin / getYBin (src/serial/DataFormats/LayerTilesSerial.h:24-40):
 * (v - minX) * rX in float, truncated, clamped to [0, 99]. */
static int o2_bin(float v) {
  const float minv = -250.f;
  const float r = 100.f / 500.f; /* nColumns / (maxX - minX) */
  int b = sat_f2i((v - minv) * r);
  if (b > O2_NCOLS - 1) b = O2_NCOLS - 1;
  if (b < 0) b = 0;
  return b;
}

typedef struct {
  int32_t *tile_start; /* O2_NLAYERS * O2_NTILES + 1 */
  int32_t *order;      /* points by (layer, tile), index order inside a tile */
  int32_t *key;
  int32_t *fstart;     /* follower lists (CSR over nearestHigher) */
  int32_t *flist;
  int32_t *stack;
  int64_t cap;
} o2_ws;

static void o2_ws_free(o2_ws *w) {
  free(w->tile_start);
  free(w->order);
  free(w->key);
  free(w->fstart);
  free(w->flist);
  free(w->stack);
  memset(w, 0, sizeof(*w));
}

static int o2_ws_reserve(o2_ws *w, int64_t n) {
  if (!w->tile_start) {
    w->tile_start = (int32_t *)malloc(sizeof(int32_t) * ((size_t)O2_NLAYERS * O2_NTILES + 1));
    if (!w->tile_start) return -1;
  }
  if (w->order && n <= w->cap) return 0;
  free(w->order);
  free(w->key);
  free(w->fstart);
  free(w->flist);
  free(w->stack);
  w->order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  w->key = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  w->fstart = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 2));
  w->flist = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  w->stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  if (!w->order || !w->key || !w->fstart || !w->flist || !w->stack) return -1;
  w->cap = n;
  return 0;
}

/* kernel_compute_histogram (src/serial/plugin-CLUEClusterizer/CLUEAlgoKernels.h:18-23):
 * every point is appended to its tile in index order.  Restated as a stable
 * counting sort into one CSR over (layer, global bin = xBin + 100*yBin). */
static void o2_fill_tiles(o2_ws *w, int32_t n, const float *x, const float *y, const int32_t *layer) {
  const int64_t nk = (int64_t)O2_NLAYERS * O2_NTILES;
  memset(w->tile_start, 0, sizeof(int32_t) * (size_t)(nk + 1));
  for (int32_t i = 0; i < n; ++i) {
    int k = layer[i] * O2_NTILES + o2_bin(x[i]) + O2_NCOLS * o2_bin(y[i]);
    w->key[i] = k;
    w->tile_start[k + 1]++;
  }
  for (int64_t k = 0; k < nk; ++k) w->tile_start[k + 1] += w->tile_start[k];
  /* stable placement: reuse fstart as a cursor copy would need nk ints, so
   * walk keys and use tile_start[k] as the running cursor, then shift back */
  for (int32_t i = 0; i < n; ++i) w->order[w->tile_start[w->key[i]]++] = i;
  for (int64_t k = nk; k > 0; --k) w->tile_start[k] = w->tile_start[k - 1];
  w->tile_start[0] = 0;
}

/* Reference distance(): sqrt(dx*dx + dy*dy) in float, same layer only
 * (CLUEAlgoKernels.h:7-16).  Callers only pass same-layer pairs. */
static float o2_dist(const float *x, const float *y, int32_t i, int32_t j) {
  const float dx = x[i] - x[j];
  const float dy = y[i] - y[j];
  return sqrtf(dx * dx + dy * dy);
}

/* kernel_calculate_density (CLUEAlgoKernels.h:25-55) */
static void o2_density(const o2_ws *w, int32_t n, const float *x, const float *y, const int32_t *layer,
                       const float *weight, float dc, float *rho) {
  for (int32_t i = 0; i < n; ++i) {
    const int32_t *ts = w->tile_start + (int64_t)layer[i] * O2_NTILES;
    int bx0 = o2_bin(x[i] - dc), bx1 = o2_bin(x[i] + dc);
    int by0 = o2_bin(y[i] - dc), by1 = o2_bin(y[i] + dc);
    float r = 0.f;
    for (int bx = bx0; bx < bx1 + 1; ++bx)
      for (int by = by0; by < by1 + 1; ++by) {
        int t = bx + O2_NCOLS * by;
        for (int32_t s = ts[t]; s < ts[t + 1]; ++s) {
          int32_t j = w->order[s];
          float d = o2_dist(x, y, i, j);
          if (d <= dc) r += (i == j ? 1.f : 0.5f) * weight[j];
        }
      }
    rho[i] = r;
  }
}

/* kernel_calculate_distanceToHigher (CLUEAlgoKernels.h:57-106) */
static void o2_nearest_higher(const o2_ws *w, int32_t n, const float *x, const float *y, const int32_t *layer,
                              const float *rho, float odf, float dc, float *delta, int32_t *nh) {
  const float dm = odf * dc;
  for (int32_t i = 0; i < n; ++i) {
    float delta_i = FLT_MAX;
    int32_t nh_i = -1;
    const float xi = x[i], yi = y[i], rho_i = rho[i];
    const int32_t *ts = w->tile_start + (int64_t)layer[i] * O2_NTILES;
    int bx0 = o2_bin(xi - dm), bx1 = o2_bin(xi + dm);
    int by0 = o2_bin(yi - dm), by1 = o2_bin(yi + dm);
    for (int bx = bx0; bx < bx1 + 1; ++bx)
      for (int by = by0; by < by1 + 1; ++by) {
        int t = bx + O2_NCOLS * by;
        for (int32_t s = ts[t]; s < ts[t + 1]; ++s) {
          int32_t j = w->order[s];
          int higher = (rho[j] > rho_i) || ((rho[j] == rho_i) && (j > i));
          float d = o2_dist(x, y, i, j);
          if (higher && d <= dm) {
            if (d < delta_i) {
              delta_i = d;
              nh_i = j;
            }
          }
        }
      }
    delta[i] = delta_i;
    nh[i] = nh_i;
  }
}

/* kernel_findAndAssign_clusters (CLUEAlgoKernels.h:108-153): seeds numbered
 * in index order, followers appended to their nearest higher in index order,
 * labels pushed down from the seeds with a LIFO stack. */
static void o2_assign(o2_ws *w, int32_t n, const float *rho, const float *delta, const int32_t *nh, float odf,
                      float dc, float rhoc, int32_t *isSeed, int32_t *clusterIndex) {
  const float dm = odf * dc;
  int32_t *fs = w->fstart;
  memset(fs, 0, sizeof(int32_t) * (size_t)(n + 2));
  int32_t nClusters = 0, top = 0;
  for (int32_t i = 0; i < n; ++i) {
    clusterIndex[i] = -1;
    isSeed[i] = 0;
    int seed = (delta[i] > dc) && (rho[i] >= rhoc);
    int outlier = (delta[i] > dm) && (rho[i] < rhoc);
    if (!seed && !outlier && nh[i] >= 0) fs[nh[i] + 2]++;
  }
  for (int32_t i = 0; i < n; ++i) fs[i + 2] += fs[i + 1];
  for (int32_t i = 0; i < n; ++i) {
    int seed = (delta[i] > dc) && (rho[i] >= rhoc);
    int outlier = (delta[i] > dm) && (rho[i] < rhoc);
    if (seed) {
      isSeed[i] = 1;
      clusterIndex[i] = nClusters++;
      w->stack[top++] = i;
    } else if (!outlier && nh[i] >= 0) {
      w->flist[fs[nh[i] + 1]++] = i;
    }
  }
  /* fs[p+1] is now the end of p's list and fs[p] its start */
  while (top > 0) {
    int32_t i = w->stack[--top];
    for (int32_t s = (i == 0 ? 0 : fs[i]); s < fs[i + 1]; ++s) {
      int32_t j = w->flist[s];
      clusterIndex[j] = clusterIndex[i];
      w->stack[top++] = j;
    }
  }
}

static int o2_run(o2_ws *w, int32_t n, const float *x, const float *y, const int32_t *layer, const float *weight,
                  float dc, float rhoc, float odf, float *rho, float *delta, int32_t *nh, int32_t *isSeed,
                  int32_t *clusterIndex) {
  if (n < 0) return -1;
  for (int32_t i = 0; i < n; ++i)
    if (layer[i] < 0 || layer[i] >= O2_NLAYERS) return -2;
  if (o2_ws_reserve(w, n)) return -3;
  o2_fill_tiles(w, n, x, y, layer);
  o2_density(w, n, x, y, layer, weight, dc, rho);
  o2_nearest_higher(w, n, x, y, layer, rho, odf, dc, delta, nh);
  o2_assign(w, n, rho, delta, nh, odf, dc, rhoc, isSeed, clusterIndex);
  return 0;
}

/* One event (CLUEAlgoSerial::makeClusters, CLUEAlgoSerial.cc:18-35).
 * Returns 0, or <0 for n<0 / a layer outside [0,100) / out of memory. */
int oracle_clue2d(int32_t n, const float *x, const float *y, const int32_t *layer, const float *weight, float dc,
                  float rhoc, float odf, float *rho, float *delta, int32_t *nearestHigher, int32_t *isSeed,
                  int32_t *clusterIndex) {
  o2_ws w;
  memset(&w, 0, sizeof(w));
  int rc = o2_run(&w, n, x, y, layer, weight, dc, rhoc, odf, rho, delta, nearestHigher, isSeed, clusterIndex);
  o2_ws_free(&w);
  return rc;
}

/* Many events over host threads, one workspace per thread: the reference's
 * EDM streams (src/serial/bin/EventProcessor.cc:33-35) without TBB.  Event e
 * is [offsets[e], offsets[e+1]) of the concatenated arrays; indices in
 * nearestHigher are event-local, as in the reference. */
typedef struct {
  int32_t n_events;
  const int64_t *off;
  const float *x, *y, *w;
  const int32_t *layer;
  float dc, rhoc, odf;
  float *rho, *delta;
  int32_t *nh, *seed, *ci;
  int32_t next;
  int32_t rc;
  pthread_mutex_t mu;
} o2_batch;

static void *o2_batch_worker(void *arg) {
  o2_batch *b = (o2_batch *)arg;
  o2_ws w;
  memset(&w, 0, sizeof(w));
  for (;;) {
    pthread_mutex_lock(&b->mu);
    int32_t e = b->next++;
    pthread_mutex_unlock(&b->mu);
    if (e >= b->n_events) break;
    int64_t s = b->off[e];
    int32_t n = (int32_t)(b->off[e + 1] - s);
    int rc = o2_run(&w, n, b->x + s, b->y + s, b->layer + s, b->w + s, b->dc, b->rhoc, b->odf, b->rho + s,
                    b->delta + s, b->nh + s, b->seed + s, b->ci + s);
    if (rc) {
      pthread_mutex_lock(&b->mu);
      b->rc = rc;
      pthread_mutex_unlock(&b->mu);
    }
  }
  o2_ws_free(&w);
  return NULL;
}

int oracle_clue2d_batch(int32_t n_events, const int64_t *offsets, const float *x, const float *y,
                        const int32_t *layer, const float *weight, float dc, float rhoc, float odf, float *rho,
                        float *delta, int32_t *nearestHigher, int32_t *isSeed, int32_t *clusterIndex,
                        int32_t n_threads) {
  o2_batch b;
  memset(&b, 0, sizeof(b));
  b.n_events = n_events;
  b.off = offsets;
  b.x = x;
  b.y = y;
  b.w = weight;
  b.layer = layer;
  b.dc = dc;
  b.rhoc = rhoc;
  b.odf = odf;
  b.rho = rho;
  b.delta = delta;
  b.nh = nearestHigher;
  b.seed = isSeed;
  b.ci = clusterIndex;
  pthread_mutex_init(&b.mu, NULL);
  if (n_threads < 1) n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
  for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, o2_batch_worker, &b);
  for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&b.mu);
  return b.rc;
}

/* ------------------------------------------------------------------------- */
/* CLUE3D                                                                     */
/* ------------------------------------------------------------------------- */

/* ticl::TileConstants (src/serial/DataFormats/Common.h:9-16) */
#define O3_NETA 34
#define O3_NPHI 126
#define O3_NBINS (O3_NETA * O3_NPHI)

typedef struct {
  int32_t n_layers;               /* TileConstants::nLayers, 94 in the reference */
  int32_t density_sibling_layers; /* CLUE3DAlgoKernels.h:29 */
  float density_xy_distance_sqr;  /* :30 */
  float kernel_density_factor;    /* :31 */
  int32_t density_on_same_layer;  /* :32 */
  int32_t nh_sibling_layers;      /* :289 */
  int32_t nh_on_same_layer;       /* :290 */
  float critical_xy_distance;     /* :511 */
  float critical_z_distance_lyr;  /* :512 */
  float critical_density;         /* :513 */
  float critical_self_density;    /* :514 */
  float outlier_multiplier;       /* :515 */
} oracle3d_params;

/* reco::reduceRange for float (src/serial/DataFormats/Math/deltaPhi.h:16-23) */
static float o3_reduce_range(float x) {
  const float o2pi = (float)(1. / (2. * M_PI));
  if (fabsf(x) <= (float)M_PI) return x;
  float n = roundf(x * o2pi);
  return x - n * (float)(2. * M_PI);
}

/* TICLLayerTileT::etaBin (src/serial/DataFormats/TICLLayerTile.h:19-26) */
static int o3_eta_bin(float eta) {
  const float eta_range = 3.2f - 1.5f;
  const float r = (float)O3_NETA / eta_range;
  int b = sat_f2i((fabsf(eta) - 1.5f) * r);
  if (b < 0) b = 0;
  if (b > O3_NETA - 1) b = O3_NETA - 1;
  return b;
}

/* TICLLayerTileT::phiBin (TICLLayerTile.h:28-34): the product is in double */
static int o3_phi_bin(float phi) {
  float norm = o3_reduce_range(phi);
  const float r = (float)(O3_NPHI * M_1_PI * 0.5f);
  double v = ((double)norm + M_PI) * (double)r;
  if (v != v) return 0;
  if (v >= 2147483648.0) return INT_MAX;
  if (v < -2147483648.0) return INT_MIN;
  return (int)v;
}

static int64_t o3_key(int32_t layer, float eta, float phi) {
  return (int64_t)layer * O3_NBINS + o3_phi_bin(phi) + (int64_t)o3_eta_bin(eta) * O3_NPHI;
}

typedef struct {
  int64_t nk;
  int32_t *tile_start; /* nk + 1 */
  int32_t *order, *fstart, *flist, *stack;
  int64_t *key;
} o3_ws;

static void o3_free(o3_ws *w) {
  free(w->tile_start);
  free(w->order);
  free(w->fstart);
  free(w->flist);
  free(w->stack);
  free(w->key);
  memset(w, 0, sizeof(*w));
}

/* KernelComputeHistogramSoA (CLUE3DAlgoKernels.h:19-24); the flat key space
 * holds nLayers*nBins bins plus the 126 that an eta row of 34 reaches past
 * the last layer. */
static int o3_fill(o3_ws *w, int32_t n, const float *eta, const float *phi, const int32_t *layer, int32_t nl) {
  w->nk = (int64_t)nl * O3_NBINS + O3_NPHI + 1;
  w->tile_start = (int32_t *)calloc((size_t)(w->nk + 1), sizeof(int32_t));
  w->order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  w->key = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  w->fstart = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 2));
  w->flist = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  w->stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  if (!w->tile_start || !w->order || !w->key || !w->fstart || !w->flist || !w->stack) return -3;
  for (int32_t i = 0; i < n; ++i) {
    /* a phi that does not reduce into [-pi, pi] would index outside its
     * layer's tiles in the reference (undefined); reject it */
    int pb = o3_phi_bin(phi[i]);
    if (pb < 0 || pb > O3_NPHI) return -2;
    int64_t k = o3_key(layer[i], eta[i], phi[i]);
    if (k < 0 || k >= w->nk) return -2;
    w->key[i] = k;
    w->tile_start[k + 1]++;
  }
  for (int64_t k = 0; k < w->nk; ++k) w->tile_start[k + 1] += w->tile_start[k];
  for (int32_t i = 0; i < n; ++i) w->order[w->tile_start[w->key[i]]++] = i;
  for (int64_t k = w->nk; k > 0; --k) w->tile_start[k] = w->tile_start[k - 1];
  w->tile_start[0] = 0;
  return 0;
}

static void o3_layer_range(int32_t layer_id, int32_t sib, int32_t nl, int upper_side_shift, int32_t *lo,
                           int32_t *hi) {
  const int32_t last = nl / 2;
  int32_t mx = 2 * last - 1, mn = 0;
  if (layer_id < last) {
    mn = layer_id - sib > mn ? layer_id - sib : mn;
    mx = layer_id + sib < last - 1 ? layer_id + sib : last - 1;
  } else {
    int32_t side_lo = last + upper_side_shift;
    mn = layer_id - sib > side_lo ? layer_id - sib : side_lo;
    mx = layer_id + sib < mx ? layer_id + sib : mx;
  }
  *lo = mn;
  *hi = mx;
}

/* KernelCalculateDensitySoA (CLUE3DAlgoKernels.h:26-150) */
static void o3_density(const o3_ws *w, int32_t n, const float *z, const float *eta, const float *phi,
                       const float *roa, const float *radius, const int32_t *layer, const float *energy,
                       const int32_t *isSilicon, const oracle3d_params *p, float *rho) {
  for (int32_t i = 0; i < n; ++i) {
    int32_t lo, hi;
    o3_layer_range(layer[i], p->density_sibling_layers, p->n_layers, 0, &lo, &hi);
    const int eb = o3_eta_bin(eta[i]), pb = o3_phi_bin(phi[i]);
    const float thr = isSilicon[i] ? p->density_xy_distance_sqr : radius[i] * radius[i];
    const float r0 = roa[i] * z[i];
    float r = 0.f;
    for (int32_t cl = lo; cl <= hi; ++cl) {
      const int same = (cl == layer[i]);
      int e0 = eb - 2 > 0 ? eb - 2 : 0;
      int e1 = eb + 2 < O3_NETA ? eb + 2 : O3_NETA;
      for (int ie = e0; ie <= e1; ++ie) {
        for (int ip_it = pb - 2; ip_it <= pb + 2; ++ip_it) {
          int ip = ((ip_it % O3_NPHI + O3_NPHI) % O3_NPHI);
          int64_t t = (int64_t)cl * O3_NBINS + (int64_t)ie * O3_NPHI + ip;
          for (int32_t s = w->tile_start[t]; s < w->tile_start[t + 1]; ++s) {
            int32_t j = w->order[s];
            const float r1 = roa[j] * z[i];
            const float dphi = o3_reduce_range(phi[i] - phi[j]);
            const float a = (r0 - r1) * (r0 - r1);
            const float b = r1 * r1 * dphi * dphi;
            if (a + b < thr) {
              float f = (same && !p->density_on_same_layer) ? 0.f : 1.f;
              float add = ((i == j) ? 1.f : p->kernel_density_factor * f) * energy[j];
              r += add;
            }
          }
        }
      }
    }
    rho[i] = r;
  }
}

/* KernelComputeDistanceToHigherSoA (CLUE3DAlgoKernels.h:286-392) */
static void o3_nearest_higher(const o3_ws *w, int32_t n, const float *z, const float *eta, const float *phi,
                              const float *roa, const int32_t *layer, const float *rho,
                              const oracle3d_params *p, float *delta_t, int32_t *delta_l, int32_t *nh_layer,
                              int32_t *nh_idx) {
  for (int32_t i = 0; i < n; ++i) {
    int32_t lo, hi;
    o3_layer_range(layer[i], p->nh_sibling_layers, p->n_layers, 1, &lo, &hi);
    const int eb = o3_eta_bin(eta[i]), pb = o3_phi_bin(phi[i]);
    const float r0 = roa[i] * z[i];
    float best = FLT_MAX, best_t = FLT_MAX;
    int32_t best_l = INT_MAX, nl = -1, ni = -1;
    for (int32_t cl = lo; cl <= hi; ++cl) {
      if (!p->nh_on_same_layer && cl == layer[i]) continue;
      int e0 = eb - 1 > 0 ? eb - 1 : 0;
      int e1 = eb + 1 < O3_NETA ? eb + 1 : O3_NETA;
      for (int ie = e0; ie <= e1; ++ie) {
        for (int ip_it = pb - 1; ip_it <= pb + 1; ++ip_it) {
          int ip = ((ip_it % O3_NPHI + O3_NPHI) % O3_NPHI);
          int64_t t = (int64_t)cl * O3_NBINS + (int64_t)ie * O3_NPHI + ip;
          for (int32_t s = w->tile_start[t]; s < w->tile_start[t + 1]; ++s) {
            int32_t j = w->order[s];
            const float r1 = roa[j] * z[i];
            const float dphi = o3_reduce_range(phi[i] - phi[j]);
            const float a = (r0 - r1) * (r0 - r1);
            const float b = r1 * r1 * dphi * dphi;
            const float d = a + b;
            if (rho[j] > rho[i] && d <= best) {
              best = d;
              best_t = sqrtf(d);
              best_l = abs(cl - layer[i]);
              nl = cl;
              ni = j;
            }
          }
        }
      }
    }
    if (best != FLT_MAX) {
      delta_t[i] = best_t;
      delta_l[i] = best_l;
      nh_layer[i] = nl;
      nh_idx[i] = ni;
    } else {
      delta_t[i] = FLT_MAX;
      delta_l[i] = INT_MAX;
      nh_layer[i] = -1;
      nh_idx[i] = -1;
    }
  }
}

/* KernelFindAndAssignClustersSoA (CLUE3DAlgoKernels.h:509-580) */
static int32_t o3_assign(o3_ws *w, int32_t n, const float *radius, const float *energy, const int32_t *isSilicon,
                         const float *rho, const float *delta_t, const int32_t *delta_l, const int32_t *nh_layer,
                         const int32_t *nh_idx, const oracle3d_params *p, int32_t *isSeed,
                         int32_t *tracksterIndex) {
  int32_t *fs = w->fstart;
  memset(fs, 0, sizeof(int32_t) * (size_t)(n + 2));
  const float out_thr = p->outlier_multiplier * p->critical_xy_distance;
  char *kind = (char *)malloc((size_t)n + 1); /* 1 seed, 2 follower, 0 other */
  for (int32_t i = 0; i < n; ++i) {
    tracksterIndex[i] = -1;
    isSeed[i] = 0;
    const float dxy = isSilicon[i] ? p->critical_xy_distance : radius[i];
    int seed = (delta_t[i] > dxy || (float)delta_l[i] > p->critical_z_distance_lyr) &&
               (rho[i] >= p->critical_density) && (energy[i] / rho[i] > p->critical_self_density);
    int outlier = (delta_t[i] > out_thr) && (rho[i] < p->critical_density);
    kind[i] = seed ? 1 : (!outlier && nh_layer[i] >= 0 ? 2 : 0);
    if (kind[i] == 2) fs[nh_idx[i] + 2]++;
  }
  for (int32_t i = 0; i < n; ++i) fs[i + 2] += fs[i + 1];
  int32_t nt = 0, top = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (kind[i] == 1) {
      tracksterIndex[i] = nt++;
      isSeed[i] = 1;
      w->stack[top++] = i;
    } else if (kind[i] == 2) {
      w->flist[fs[nh_idx[i] + 1]++] = i;
    }
  }
  while (top > 0) {
    int32_t i = w->stack[--top];
    for (int32_t s = (i == 0 ? 0 : fs[i]); s < fs[i + 1]; ++s) {
      int32_t j = w->flist[s];
      tracksterIndex[j] = tracksterIndex[i];
      w->stack[top++] = j;
    }
  }
  free(kind);
  return nt;
}

/* One event of CLUE3DAlgoSerial::makeTrackstersSoA (CLUE3DAlgoSerial.cc:42-50)
 * with every default argument exposed and nLayers a parameter.  Returns the
 * number of tracksters, or <0 on bad input (layer outside [0, n_layers)). */
int oracle_clue3d(int32_t n, const float *z, const float *eta, const float *phi, const float *r_over_absz,
                  const float *radius, const int32_t *layer, const float *energy, const int32_t *isSilicon,
                  const oracle3d_params *p, float *rho, float *delta_t, int32_t *delta_l, int32_t *nh_layer,
                  int32_t *nh_idx, int32_t *isSeed, int32_t *tracksterIndex) {
  if (n < 0) return -1;
  for (int32_t i = 0; i < n; ++i)
    if (layer[i] < 0 || layer[i] >= p->n_layers) return -2;
  o3_ws w;
  memset(&w, 0, sizeof(w));
  int rc = o3_fill(&w, n, eta, phi, layer, p->n_layers);
  if (rc) {
    o3_free(&w);
    return rc;
  }
  o3_density(&w, n, z, eta, phi, r_over_absz, radius, layer, energy, isSilicon, p, rho);
  o3_nearest_higher(&w, n, z, eta, phi, r_over_absz, layer, rho, p, delta_t, delta_l, nh_layer, nh_idx);
  int32_t nt = o3_assign(&w, n, radius, energy, isSilicon, rho, delta_t, delta_l, nh_layer, nh_idx, p, isSeed,
                         tracksterIndex);
  o3_free(&w);
  return nt;
}

/* CSR batch of CLUE3D events over n_threads host threads: event e is
 * [offsets[e], offsets[e+1]) of every array; n_tracksters[e] receives the
 * event's trackster count.  Returns 0, or the first event's error code. */
typedef struct {
  int32_t n_events;
  const int64_t *off;
  const float *z, *eta, *phi, *roa, *radius, *energy;
  const int32_t *layer, *sil;
  const oracle3d_params *p;
  float *rho, *delta_t;
  int32_t *delta_l, *nh_layer, *nh_idx, *seed, *ti, *nt;
  int32_t next;
  int32_t rc;
  pthread_mutex_t mu;
} o3_batch;

static void *o3_batch_worker(void *arg) {
  o3_batch *b = (o3_batch *)arg;
  for (;;) {
    pthread_mutex_lock(&b->mu);
    int32_t e = b->next++;
    pthread_mutex_unlock(&b->mu);
    if (e >= b->n_events) break;
    int64_t s = b->off[e];
    int32_t n = (int32_t)(b->off[e + 1] - s);
    int32_t nt = oracle_clue3d(n, b->z + s, b->eta + s, b->phi + s, b->roa + s, b->radius + s, b->layer + s,
                               b->energy + s, b->sil + s, b->p, b->rho + s, b->delta_t + s, b->delta_l + s,
                               b->nh_layer + s, b->nh_idx + s, b->seed + s, b->ti + s);
    b->nt[e] = nt;
    if (nt < 0) {
      pthread_mutex_lock(&b->mu);
      if (!b->rc) b->rc = nt;
      pthread_mutex_unlock(&b->mu);
    }
  }
  return NULL;
}

int oracle_clue3d_batch(int32_t n_events, const int64_t *offsets, const float *z, const float *eta,
                        const float *phi, const float *r_over_absz, const float *radius, const int32_t *layer,
                        const float *energy, const int32_t *isSilicon, const oracle3d_params *p, float *rho,
                        float *delta_t, int32_t *delta_l, int32_t *nh_layer, int32_t *nh_idx, int32_t *isSeed,
                        int32_t *tracksterIndex, int32_t *n_tracksters, int32_t n_threads) {
  o3_batch b;
  memset(&b, 0, sizeof(b));
  b.n_events = n_events;
  b.off = offsets;
  b.z = z;
  b.eta = eta;
  b.phi = phi;
  b.roa = r_over_absz;
  b.radius = radius;
  b.energy = energy;
  b.layer = layer;
  b.sil = isSilicon;
  b.p = p;
  b.rho = rho;
  b.delta_t = delta_t;
  b.delta_l = delta_l;
  b.nh_layer = nh_layer;
  b.nh_idx = nh_idx;
  b.seed = isSeed;
  b.ti = tracksterIndex;
  b.nt = n_tracksters;
  pthread_mutex_init(&b.mu, NULL);
  if (n_threads < 1) n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
  for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, o3_batch_worker, &b);
  for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&b.mu);
  return b.rc;
}
