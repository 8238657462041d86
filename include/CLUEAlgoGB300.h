// CLUEAlgoGB300.h -- C++ adapter with the reference producer's signature.
//
// A drop-in for CLUEAlgoSerial inside CLUESerialClusterizer::produce
// (src/serial/plugin-CLUEClusterizer/CLUESerialClusterizer.cc:29-36):
//
//   CLUEAlgoGB300 algo(dc, rhoc, odf);
//   algo.makeClusters(pc, d_points, par.dc, par.rhoc, par.outlierDeltaFactor);
//
// PointsCloud / PointsCloudSerial are the reference's types
// (src/serial/DataFormats/PointsCloud.h); they are template parameters here so
// that this header needs nothing from the reference tree.  The outputs are
// bit-identical to CLUEAlgoSerial::makeClusters; `followers` is left empty
// because the GPU path resolves clusters without follower lists.
// Errors throw std::runtime_error carrying clue_last_error().
#ifndef CLUE_GB300_CLUEALGOGB300_H
#define CLUE_GB300_CLUEALGOGB300_H

#include <stdexcept>
#include <string>

#include "clue.h"

class CLUEAlgoGB300 {
 public:
  CLUEAlgoGB300(float dc, float rhoc, float outlierDeltaFactor, size_t device_budget_bytes = 0, int device = 0,
                void* cuda_stream = nullptr) {
    clue_params p{dc, rhoc, outlierDeltaFactor};
    check(clue_create(&p, device_budget_bytes, device, cuda_stream, &h_));
  }
  ~CLUEAlgoGB300() { clue_destroy(h_); }
  CLUEAlgoGB300(const CLUEAlgoGB300&) = delete;
  CLUEAlgoGB300& operator=(const CLUEAlgoGB300&) = delete;

  // CLUEAlgoSerial::makeClusters (src/serial/plugin-CLUEClusterizer/CLUEAlgoSerial.h:13)
  template <class PC, class PCS>
  void makeClusters(PC const& host_pc, PCS& d_points, float const& dc, float const& rhoc,
                    float const& outlierDeltaFactor) {
    clue_params p{dc, rhoc, outlierDeltaFactor};
    check(clue_set_params(h_, &p));
    const auto n = host_pc.x.size();
    d_points.x = host_pc.x;
    d_points.y = host_pc.y;
    d_points.layer = host_pc.layer;
    d_points.weight = host_pc.weight;
    d_points.rho.resize(n);
    d_points.delta.resize(n);
    d_points.nearestHigher.resize(n);
    d_points.isSeed.resize(n);
    d_points.clusterIndex.resize(n);
    d_points.followers.clear();
    clue_outputs out{d_points.rho.data(), d_points.delta.data(), d_points.nearestHigher.data(),
                     d_points.isSeed.data(), d_points.clusterIndex.data()};
    check(clue_run_event(h_, static_cast<int32_t>(n), host_pc.x.data(), host_pc.y.data(), host_pc.layer.data(),
                         host_pc.weight.data(), &out, CLUE_HOST_MEMORY));
  }

  clue_handle* handle() const { return h_; }

 private:
  static void check(int rc) {
    if (rc != CLUE_OK) throw std::runtime_error(std::string("clue: ") + clue_last_error());
  }
  clue_handle* h_ = nullptr;
};

#endif  // CLUE_GB300_CLUEALGOGB300_H
