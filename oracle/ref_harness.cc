// Test infrastructure, not product code.
//
// C entry points around the UNMODIFIED serial CLUE sources of
// tonydp03/heterogeneous-clue.  Nothing from the reference is copied here:
// the two algorithm translation units are #included from the reference tree
// at build time (oracle/build.py passes -I <reference>/src/serial), and the
// result goes to oracle/_ref/libclue_ref.so, which stays out of git.
//
// Used only by tests/ (to pin the CPU restatement in oracle/clue_oracle.c)
// and by tests/golden/make_golden.py (to write the golden vectors).  Build
// flags: -std=c++17 -O2 -ffp-contract=off, without the reference Makefile's
// -mavx/-march=native (x86-only, and FMA contraction changes delta bits).
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "plugin-CLUEClusterizer/CLUEAlgoSerial.cc"
#include "plugin-CLUETracksterizer/CLUE3DAlgoSerial.cc"

extern "C" {

// CLUEAlgoSerial::makeClusters (src/serial/plugin-CLUEClusterizer/CLUEAlgoSerial.cc:18-35)
// on one event.  Returns 0.
int ref_clue2d(int32_t n, const float* x, const float* y, const int32_t* layer, const float* weight,
               float dc, float rhoc, float odf,
               float* rho, float* delta, int32_t* nearestHigher, int32_t* isSeed, int32_t* clusterIndex) {
  PointsCloud pc;
  pc.x.assign(x, x + n);
  pc.y.assign(y, y + n);
  pc.layer.assign(layer, layer + n);
  pc.weight.assign(weight, weight + n);
  CLUEAlgoSerial algo;
  PointsCloudSerial out;
  algo.makeClusters(pc, out, dc, rhoc, odf);
  for (int32_t i = 0; i < n; ++i) {
    rho[i] = out.rho[i];
    delta[i] = out.delta[i];
    nearestHigher[i] = out.nearestHigher[i];
    isSeed[i] = out.isSeed[i];
    clusterIndex[i] = out.clusterIndex[i];
  }
  return 0;
}

// CLUEAlgoSerial::makeClusters over a CSR batch of events (event e is
// [offsets[e], offsets[e+1]) of every array) on n_threads host threads, one
// CLUEAlgoSerial per thread reused for all of its events, as the reference
// runs one producer, hence one algorithm object, per EDM stream
// (src/serial/bin/StreamSchedule.cc:15-39, CLUESerialClusterizer.cc:29-36).
// Each event's PointsCloud is built before the clock starts and its outputs
// are copied out after it stops, so *seconds is the wall time of the
// makeClusters calls alone (their own setup copy and tile clearing included).
// Events are handed out in order from a shared counter.  Returns 0.
int ref_clue2d_batch(int32_t n_events, const int64_t* offsets, const float* x, const float* y,
                     const int32_t* layer, const float* weight, float dc, float rhoc, float odf, float* rho,
                     float* delta, int32_t* nearestHigher, int32_t* isSeed, int32_t* clusterIndex,
                     int32_t n_threads, double* seconds) {
  std::vector<PointsCloud> in(n_events);
  std::vector<PointsCloudSerial> out(n_events);
  for (int32_t e = 0; e < n_events; ++e) {
    const int64_t s = offsets[e], t = offsets[e + 1];
    in[e].x.assign(x + s, x + t);
    in[e].y.assign(y + s, y + t);
    in[e].layer.assign(layer + s, layer + t);
    in[e].weight.assign(weight + s, weight + t);
  }
  if (n_threads < 1) n_threads = 1;
  // the algorithm objects (each 100 x 10,000 tiles) exist before the clock starts
  std::vector<std::unique_ptr<CLUEAlgoSerial>> algos;
  for (int32_t t = 0; t < n_threads; ++t) algos.emplace_back(new CLUEAlgoSerial);
  std::atomic<int32_t> next{0};
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (int32_t t = 0; t < n_threads; ++t) {
    th.emplace_back([&, t]() {
      for (int32_t e; (e = next.fetch_add(1)) < n_events;) algos[t]->makeClusters(in[e], out[e], dc, rhoc, odf);
    });
  }
  for (auto& t : th) t.join();
  const auto t1 = std::chrono::steady_clock::now();
  *seconds = std::chrono::duration<double>(t1 - t0).count();
  for (int32_t e = 0; e < n_events; ++e) {
    const int64_t s = offsets[e];
    const size_t n = out[e].rho.size();
    for (size_t i = 0; i < n; ++i) {
      rho[s + i] = out[e].rho[i];
      delta[s + i] = out[e].delta[i];
      nearestHigher[s + i] = out[e].nearestHigher[i];
      isSeed[s + i] = out[e].isSeed[i];
      clusterIndex[s + i] = out[e].clusterIndex[i];
    }
  }
  return 0;
}

// The four SoA stages of CLUE3DAlgoSerial::makeTrackstersSoA
// (src/serial/plugin-CLUETracksterizer/CLUE3DAlgoSerial.cc:42-50), called
// directly so that the default arguments of
// src/serial/plugin-CLUETracksterizer/CLUE3DAlgoKernels.h:26-32,286-290,509-515
// can be overridden.  The tile geometry stays the reference's (94 layers):
// callers must keep layer < 94.
int ref_clue3d(int32_t n, const float* z, const float* eta, const float* phi, const float* r_over_absz,
               const float* radius, const int32_t* layer, const float* energy, const int32_t* isSilicon,
               int32_t densitySiblingLayers, float densityXYDistanceSqr, float kernelDensityFactor,
               int32_t densityOnSameLayer, int32_t nhSiblingLayers, int32_t nearestHigherOnSameLayer,
               float criticalXYDistance, float criticalZDistanceLyr, float criticalDensity,
               float criticalSelfDensity, float outlierMultiplier,
               float* rho, float* delta_t, int32_t* delta_l, int32_t* nh_layer, int32_t* nh_idx,
               int32_t* isSeed, int32_t* tracksterIndex, int32_t* nTracksters) {
  ClusterCollectionSerial pts;
  pts.x.assign(n, 0.f);
  pts.y.assign(n, 0.f);
  pts.z.assign(z, z + n);
  pts.eta.assign(eta, eta + n);
  pts.phi.assign(phi, phi + n);
  pts.r_over_absz.assign(r_over_absz, r_over_absz + n);
  pts.radius.assign(radius, radius + n);
  pts.layer.assign(layer, layer + n);
  pts.energy.assign(energy, energy + n);
  pts.isSilicon.assign(isSilicon, isSilicon + n);
  pts.outResize();
  std::unique_ptr<TICLLayerTiles> hist(new TICLLayerTiles);
  KernelComputeHistogramSoA(*hist, pts);
  KernelCalculateDensitySoA(*hist, pts, 0, densitySiblingLayers, densityXYDistanceSqr, kernelDensityFactor,
                            densityOnSameLayer != 0);
  KernelComputeDistanceToHigherSoA(*hist, pts, 0, nhSiblingLayers, nearestHigherOnSameLayer != 0);
  int nt = KernelFindAndAssignClustersSoA(pts, 0, criticalXYDistance, criticalZDistanceLyr, criticalDensity,
                                          criticalSelfDensity, outlierMultiplier);
  for (int32_t i = 0; i < n; ++i) {
    rho[i] = pts.rho[i];
    delta_t[i] = pts.delta[i].first;
    delta_l[i] = pts.delta[i].second;
    nh_layer[i] = pts.nearestHigher[i].first;
    nh_idx[i] = pts.nearestHigher[i].second;
    isSeed[i] = pts.isSeed[i];
    tracksterIndex[i] = pts.tracksterIndex[i];
  }
  *nTracksters = nt;
  return 0;
}

}  // extern "C"
