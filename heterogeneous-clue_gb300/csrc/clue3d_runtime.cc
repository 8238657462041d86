// Host side of CLUE3D: parameters, buffers and the clue3d_* C entry points.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/clue.h"
#include "clue_internal.h"
#include "clue_runtime.h"

namespace clue {
namespace {

constexpr int kEta = 34;
constexpr int kPhi = 126;

// Binning constants evaluated exactly as the reference's constexpr code does
// (src/serial/DataFormats/TICLLayerTile.h:20-31, src/serial/DataFormats/Math/deltaPhi.h:18-22).
Params3D make_params3d(const clue3d_params& q) {
  Params3D p;
  p.n_layers = q.n_layers;
  p.dens_sib = q.density_sibling_layers;
  p.nh_sib = q.nh_sibling_layers;
  p.dens_same = q.density_on_same_layer;
  p.nh_same = q.nh_on_same_layer;
  p.dens_thr = q.density_xy_distance_sqr;
  p.kdf = q.kernel_density_factor;
  p.crit_xy = q.critical_xy_distance;
  p.crit_z = q.critical_z_distance_lyr;
  p.crit_rho = q.critical_density;
  p.crit_self = q.critical_self_density;
  p.outlier_mult = q.outlier_multiplier;
  volatile float om = q.outlier_multiplier, cx = q.critical_xy_distance;
  p.out_thr = om * cx;
  volatile float max_eta = 3.2f, min_eta = 1.5f;
  const float eta_range = max_eta - min_eta;
  volatile float nbins = (float)kEta;
  p.eta_r = nbins / eta_range;
  p.phi_r = (float)(kPhi * M_1_PI * 0.5f);
  p.o2pi = (float)(1. / (2. * M_PI));
  p.pi_f = (float)M_PI;
  p.twopi_f = (float)(2. * M_PI);
  return p;
}

enum Slot3D : int {
  T_OFF, T_BEV, T_KEY, T_RCNT, T_RSTART, T_ARR, T_SORTED, T_SCOL, T_TMP, T_PAR, T_EVSEEDS, T_FLAGS, T_MASK, T_REP, T_CAND, T_QREC, T_TCAND, T_TQREC,
  T_IN0, T_IN1, T_IN2, T_IN3, T_IN4, T_IN5, T_IN6, T_IN7,
  T_OUT0, T_OUT1, T_OUT2, T_OUT3, T_OUT4, T_OUT5, T_OUT6,
  T_COUNT
};

}  // namespace
}  // namespace clue

using namespace clue;

extern "C" {

void clue3d_default_params(clue3d_params* p) {
  if (!p) return;
  // src/serial/DataFormats/Common.h:14 and the default arguments of
  // src/serial/plugin-CLUETracksterizer/CLUE3DAlgoKernels.h:26-32,286-290,509-515
  p->n_layers = 94;
  p->density_sibling_layers = 3;
  p->density_xy_distance_sqr = 3.24f;
  p->kernel_density_factor = 0.2f;
  p->density_on_same_layer = 0;
  p->nh_sibling_layers = 3;
  p->nh_on_same_layer = 0;
  p->critical_xy_distance = 1.8f;
  p->critical_z_distance_lyr = 5.f;
  p->critical_density = 0.6f;
  p->critical_self_density = 0.15f;
  p->outlier_multiplier = 2.f;
}

int clue3d_run_batch(clue_handle* hh, const clue3d_params* prm, int32_t E, const int64_t* off,
                     const clue3d_inputs* in, const clue3d_outputs* out, int32_t* n_tracksters, int flags) {
  return clue::guarded([&]() -> int {
    if (!hh || !prm || !in || !out) return set_error(CLUE_EINVAL, "NULL argument");
    if (E < 0) return set_error(CLUE_EINVAL, "n_events < 0");
    if (E == 0) return CLUE_OK;
    if (!off || off[0] != 0) return set_error(CLUE_EINVAL, "event_offsets must start at 0");
    for (int32_t e = 0; e < E; ++e)
      if (off[e + 1] < off[e]) return set_error(CLUE_EINVAL, "event_offsets must be non-decreasing");
    const int64_t N = off[E];
    if (N > INT32_MAX) return set_error(CLUE_EINVAL, "more than 2^31-1 layer clusters in one call");
    if (prm->n_layers < 1 || prm->n_layers > 1000) return set_error(CLUE_EINVAL, "n_layers must be in [1, 1000]");
    const int64_t n_rows = (int64_t)prm->n_layers * kEta + 2;
    if ((int64_t)E * n_rows >= INT32_MAX) return set_error(CLUE_EINVAL, "too many events for one call");
    if (N == 0) {
      if (n_tracksters)
        for (int32_t e = 0; e < E; ++e) n_tracksters[e] = 0;
      return CLUE_OK;
    }
    const void* ins[8] = {in->z, in->eta, in->phi, in->r_over_absz, in->radius, in->layer, in->energy, in->isSilicon};
    void* outs[7] = {out->rho, out->delta_transverse, out->delta_layers, out->nh_layer, out->nh_index, out->isSeed,
                     out->tracksterIndex};
    for (auto p : ins)
      if (!p) return set_error(CLUE_EINVAL, "NULL input array");
    for (auto p : outs)
      if (!p) return set_error(CLUE_EINVAL, "NULL output array");

    Handle* h = reinterpret_cast<Handle*>(hh);
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    int rc = h->wait_previous();
    if (rc) return rc;
    const bool host_io = !(flags & CLUE_DEVICE_MEMORY);
    std::vector<size_t> need(T_COUNT, 0);
    need[T_OFF] = 8 * (size_t)(E + 1);
    const int64_t n_blk = (N + 255) / 256;
    need[T_BEV] = 4 * (size_t)n_blk;
    need[T_KEY] = need[T_ARR] = need[T_SORTED] = need[T_SCOL] = need[T_TMP] = need[T_PAR] = 4 * (size_t)N;
    need[T_RCNT] = 4 * (size_t)(E * n_rows);
    need[T_RSTART] = 4 * (size_t)(E * n_rows + 1);
    need[T_EVSEEDS] = 4 * (size_t)E;
    need[T_FLAGS] = 4 * kFlagCount;
    need[T_MASK] = need[T_REP] = 16 * (size_t)(E * n_rows);
    need[T_CAND] = need[T_QREC] = need[T_TCAND] = need[T_TQREC] = 16 * (size_t)N;
    if (host_io) {
      for (int s = T_IN0; s <= T_OUT6; ++s) need[s] = 4 * (size_t)N;
    }
    rc = h->arena3d.reserve(need, h->budget > h->arena.total() ? h->budget - h->arena.total() : 0);
    if (rc) return rc;
    rc = h->stage.reserve(8 * (size_t)(E + 1) + 4 * (size_t)n_blk);
    if (rc) return rc;
    rc = h->flags_host.reserve(4 * kFlagCount);
    if (rc) return rc;
    rc = h->nt_host.reserve(4 * (size_t)E);
    if (rc) return rc;
    memcpy(h->stage.p, off, 8 * (size_t)(E + 1));
    // the event of each 256-cluster block's first cluster, so that a kernel
    // finds a cluster's event in a step or two instead of a binary search
    int32_t* bev = reinterpret_cast<int32_t*>(static_cast<char*>(h->stage.p) + 8 * (size_t)(E + 1));
    for (int64_t j = 0, ev = 0; j < n_blk; ++j) {
      while (off[ev + 1] <= 256 * j) ++ev;
      bev[j] = (int32_t)ev;
    }

    auto P = [&](int s) { return h->arena3d.ptr(s); };
    cudaStream_t s = h->stream;
    Batch3D b;
    b.n_events = E;
    b.n_points = N;
    b.n_rows = (int32_t)n_rows;
    b.offsets = static_cast<const int64_t*>(P(T_OFF));
    const void* din[8];
    void* dout[7];
    const size_t n4 = 4 * (size_t)N;
    if ((e = cudaMemsetAsync(P(T_FLAGS), 0, 4 * kFlagCount, s)) != cudaSuccess) return cuda_error(e, "memset");
    if ((e = cudaMemcpyAsync(P(T_OFF), h->stage.p, 8 * (size_t)(E + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P(T_BEV), bev, 4 * (size_t)n_blk, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_error(e, "H2D offsets");
    b.blk_ev = static_cast<const int32_t*>(P(T_BEV));
    for (int i = 0; i < 8; ++i) {
      if (host_io) {
        din[i] = P(T_IN0 + i);
        if ((e = cudaMemcpyAsync(P(T_IN0 + i), ins[i], n4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
          return cuda_error(e, "H2D layer clusters");
      } else {
        din[i] = ins[i];
      }
    }
    for (int i = 0; i < 7; ++i) dout[i] = host_io ? P(T_OUT0 + i) : outs[i];
    b.z = static_cast<const float*>(din[0]);
    b.eta = static_cast<const float*>(din[1]);
    b.phi = static_cast<const float*>(din[2]);
    b.roa = static_cast<const float*>(din[3]);
    b.radius = static_cast<const float*>(din[4]);
    b.layer = static_cast<const int32_t*>(din[5]);
    b.energy = static_cast<const float*>(din[6]);
    b.sil = static_cast<const int32_t*>(din[7]);
    b.rho = static_cast<float*>(dout[0]);
    b.delta_t = static_cast<float*>(dout[1]);
    b.delta_l = static_cast<int32_t*>(dout[2]);
    b.nh_l = static_cast<int32_t*>(dout[3]);
    b.nh_i = static_cast<int32_t*>(dout[4]);
    b.seed = static_cast<int32_t*>(dout[5]);
    b.ti = static_cast<int32_t*>(dout[6]);
    b.key = static_cast<int32_t*>(P(T_KEY));
    b.row_cnt = static_cast<int32_t*>(P(T_RCNT));
    b.row_start = static_cast<int32_t*>(P(T_RSTART));
    b.arr = static_cast<int32_t*>(P(T_ARR));
    b.sorted = static_cast<int32_t*>(P(T_SORTED));
    b.scol = static_cast<int32_t*>(P(T_SCOL));
    b.tmp = static_cast<int32_t*>(P(T_TMP));
    b.par = static_cast<int32_t*>(P(T_PAR));
    b.ev_seeds = static_cast<int32_t*>(P(T_EVSEEDS));
    b.flags = static_cast<int32_t*>(P(T_FLAGS));
    b.row_mask = static_cast<unsigned long long*>(P(T_MASK));
    b.row_rep = static_cast<unsigned long long*>(P(T_REP));
    b.cand = static_cast<float4*>(P(T_CAND));
    b.qrec = static_cast<float4*>(P(T_QREC));
    b.tcand = static_cast<float4*>(P(T_TCAND));
    b.tqrec = static_cast<float4*>(P(T_TQREC));
    e = launch_clue3d(b, make_params3d(*prm), s);
    if (e != cudaSuccess) return cuda_error(e, "launching CLUE3D kernels");
    if (host_io) {
      for (int i = 0; i < 7; ++i)
        if ((e = cudaMemcpyAsync(outs[i], dout[i], n4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
          return cuda_error(e, "D2H outputs");
    }
    if ((e = cudaMemcpyAsync(h->nt_host.p, b.ev_seeds, 4 * (size_t)E, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->flags_host.p, b.flags, 4 * kFlagCount, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_error(e, "D2H status");
    if ((e = cudaEventRecord(h->done_event, s)) != cudaSuccess) return cuda_error(e, "cudaEventRecord");
    h->pending = true;
    h->error_layers = prm->n_layers;
    if (host_io) {
      rc = h->wait_previous();
      if (rc) return rc;
      const int32_t* f = static_cast<const int32_t*>(h->flags_host.p);
      if (f[kFlagError] == 2) {
        static_cast<int32_t*>(h->flags_host.p)[kFlagError] = 0;
        return set_error(CLUE_EINVAL, "a layer cluster's phi does not reduce into [-pi, pi]");
      }
      rc = h->check_device_flags();
      if (rc) return rc;
      if (n_tracksters) memcpy(n_tracksters, h->nt_host.p, 4 * (size_t)E);
    }
    return CLUE_OK;
  });
}

}  // extern "C"
