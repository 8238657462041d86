// CLUEAlgoGB300CUDA.h -- device-resident adapter with the reference CUDA
// producer's signature.
//
// A drop-in for CLUEAlgoCUDA inside CLUECUDAClusterizer::produce
// (src/cuda/plugin-CLUEClusterizer/CLUECUDAClusterizer.cc:31-41):
//
//   PointsCloudCUDA d_points(stream, pc.x.size());
//   if (!algo) algo = std::make_unique<CLUEAlgoGB300CUDA>(par.dc, par.rhoc, par.outlierDeltaFactor, stream);
//   algo->makeClusters(pc, d_points, stream);
//
// The inputs are copied into the caller's device buffers and the results stay
// there (rho, delta, nearestHigher, isSeed, clusterIndex), as in the
// reference's Product<PointsCloudCUDA>.  transferToHost() is the D2H step of the
// reference's CUDA CLUEOutputProducer
// (src/cuda/plugin-CLUEOutputProducer/CLUEOutputProducer.cc:36-66).
//
// PointsCloud / PointsCloudCUDA are template parameters: any types whose
// members x, y, layer, weight, rho, delta, nearestHigher, isSeed, clusterIndex
// are host vectors (PointsCloud) or expose .get() device pointers
// (PointsCloudCUDA) fit.  Results are bit-identical to CLUEAlgoSerial.
// Errors throw std::runtime_error carrying clue_last_error().
#ifndef CLUE_GB300_CLUEALGOGB300CUDA_H
#define CLUE_GB300_CLUEALGOGB300CUDA_H

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "clue.h"

class CLUEAlgoGB300CUDA {
 public:
  // CLUEAlgoCUDA(dc, rhoc, outlierDeltaFactor, stream)
  // (src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.h:14-17)
  CLUEAlgoGB300CUDA(float const& dc, float const& rhoc, float const& outlierDeltaFactor, cudaStream_t stream,
                    size_t device_budget_bytes = 0, int device = 0) {
    clue_params p{dc, rhoc, outlierDeltaFactor};
    check(clue_create(&p, device_budget_bytes, device, stream, &h_));
  }
  ~CLUEAlgoGB300CUDA() { clue_destroy(h_); }
  CLUEAlgoGB300CUDA(const CLUEAlgoGB300CUDA&) = delete;
  CLUEAlgoGB300CUDA& operator=(const CLUEAlgoGB300CUDA&) = delete;

  // CLUEAlgoCUDA::makeClusters (src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.cu:59-81):
  // H2D of the inputs on `stream`, the clustering on the device, results left
  // in d_points.  Like the reference, it returns once the stream has finished.
  template <class PC, class PCC>
  void makeClusters(PC const& host_pc, PCC& d_points, cudaStream_t stream) {
    const size_t n = host_pc.x.size();
    check(clue_set_stream(h_, stream));
    copy(d_points.x.get(), host_pc.x.data(), 4 * n, cudaMemcpyHostToDevice, stream);
    copy(d_points.y.get(), host_pc.y.data(), 4 * n, cudaMemcpyHostToDevice, stream);
    copy(d_points.layer.get(), host_pc.layer.data(), 4 * n, cudaMemcpyHostToDevice, stream);
    copy(d_points.weight.get(), host_pc.weight.data(), 4 * n, cudaMemcpyHostToDevice, stream);
    clue_outputs out{d_points.rho.get(), d_points.delta.get(), d_points.nearestHigher.get(), d_points.isSeed.get(),
                     d_points.clusterIndex.get()};
    check(clue_run_event(h_, static_cast<int32_t>(n), d_points.x.get(), d_points.y.get(), d_points.layer.get(),
                         d_points.weight.get(), &out, CLUE_DEVICE_MEMORY));
    check(clue_synchronize(h_));
  }

  // The D2H of the CUDA CLUEOutputProducer: results.outResize() then one copy
  // per output column, then a stream synchronisation.
  template <class PCC, class PC>
  static void transferToHost(PCC const& d_points, PC& results, cudaStream_t stream) {
    results.outResize();
    const size_t n = results.x.size();
    copy(results.rho.data(), d_points.rho.get(), 4 * n, cudaMemcpyDeviceToHost, stream);
    copy(results.delta.data(), d_points.delta.get(), 4 * n, cudaMemcpyDeviceToHost, stream);
    copy(results.nearestHigher.data(), d_points.nearestHigher.get(), 4 * n, cudaMemcpyDeviceToHost, stream);
    copy(results.isSeed.data(), d_points.isSeed.get(), 4 * n, cudaMemcpyDeviceToHost, stream);
    copy(results.clusterIndex.data(), d_points.clusterIndex.get(), 4 * n, cudaMemcpyDeviceToHost, stream);
    cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  }

  clue_handle* handle() const { return h_; }

 private:
  static void check(int rc) {
    if (rc != CLUE_OK) throw std::runtime_error(std::string("clue: ") + clue_last_error());
  }
  static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("clue: ") + what + ": " + cudaGetErrorString(e));
  }
  static void copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    if (bytes) cuda_check(cudaMemcpyAsync(dst, src, bytes, kind, s), "cudaMemcpyAsync");
  }
  clue_handle* h_ = nullptr;
};

#endif  // CLUE_GB300_CLUEALGOGB300CUDA_H
