// Test driver for the two C++ adapters (include/CLUEAlgoGB300.h and
// include/CLUEAlgoGB300CUDA.h), written the way the reference's producers call
// CLUEAlgoSerial and CLUEAlgoCUDA.
//
//   adapter_demo <raw2D file> <output file> <dc> <rhoc> <odf>
//
// Reads every event of a raw2D file (uint32 n, then n {x, y, layer, weight}
// float records), runs each through both adapters and writes, per event and
// per adapter, n followed by the columns rho, delta, nearestHigher, isSeed,
// clusterIndex (4 bytes each).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "CLUEAlgoGB300.h"
#include "CLUEAlgoGB300CUDA.h"

struct PointsCloud {  // the reference's host SoA (inputs and results)
  std::vector<float> x, y, weight, rho, delta;
  std::vector<int> layer, nearestHigher, isSeed, clusterIndex;
  std::vector<std::vector<int>> followers;
  void outResize() {
    auto n = x.size();
    rho.resize(n);
    delta.resize(n);
    nearestHigher.resize(n);
    clusterIndex.resize(n);
    followers.resize(n);
    isSeed.resize(n);
  }
};
using PointsCloudSerial = PointsCloud;

struct DeviceFree {
  void operator()(void* p) const { cudaFree(p); }
};
template <class T>
using dev_ptr = std::unique_ptr<T[], DeviceFree>;
template <class T>
dev_ptr<T> dev_alloc(size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
    std::fprintf(stderr, "cudaMalloc failed\n");
    std::exit(1);
  }
  return dev_ptr<T>(static_cast<T*>(p));
}

struct PointsCloudCUDA {  // device buffers owned by the caller
  explicit PointsCloudCUDA(size_t n)
      : x(dev_alloc<float>(n)), y(dev_alloc<float>(n)), layer(dev_alloc<int>(n)), weight(dev_alloc<float>(n)),
        rho(dev_alloc<float>(n)), delta(dev_alloc<float>(n)), nearestHigher(dev_alloc<int>(n)),
        clusterIndex(dev_alloc<int>(n)), isSeed(dev_alloc<int>(n)) {}
  dev_ptr<float> x, y;
  dev_ptr<int> layer;
  dev_ptr<float> weight, rho, delta;
  dev_ptr<int> nearestHigher, clusterIndex, isSeed;
};

static void put(FILE* f, const void* p, size_t bytes) {
  if (bytes && std::fwrite(p, 1, bytes, f) != bytes) {
    std::fprintf(stderr, "write failed\n");
    std::exit(1);
  }
}

static void dump(FILE* f, const PointsCloud& r) {
  uint32_t n = static_cast<uint32_t>(r.x.size());
  put(f, &n, 4);
  put(f, r.rho.data(), 4 * n);
  put(f, r.delta.data(), 4 * n);
  put(f, r.nearestHigher.data(), 4 * n);
  put(f, r.isSeed.data(), 4 * n);
  put(f, r.clusterIndex.data(), 4 * n);
}

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s raw2D out dc rhoc odf\n", argv[0]);
    return 2;
  }
  const float dc = std::strtof(argv[3], nullptr), rhoc = std::strtof(argv[4], nullptr),
              odf = std::strtof(argv[5], nullptr);
  FILE* in = std::fopen(argv[1], "rb");
  FILE* out = std::fopen(argv[2], "wb");
  if (!in || !out) return 2;
  cudaStream_t stream;
  if (cudaStreamCreate(&stream) != cudaSuccess) return 1;
  try {
    CLUEAlgoGB300 serial_algo(dc, rhoc, odf);
    std::unique_ptr<CLUEAlgoGB300CUDA> cuda_algo;
    uint32_t n;
    while (std::fread(&n, 4, 1, in) == 1) {
      std::vector<float> rec(4 * (size_t)n);
      if (std::fread(rec.data(), 16, n, in) != n) return 3;
      PointsCloud pc;
      for (uint32_t i = 0; i < n; ++i) {
        pc.x.push_back(rec[4 * i]);
        pc.y.push_back(rec[4 * i + 1]);
        pc.layer.push_back(static_cast<int>(rec[4 * i + 2]));
        pc.weight.push_back(rec[4 * i + 3]);
      }
      // CLUESerialClusterizer::produce
      PointsCloudSerial d_points;
      serial_algo.makeClusters(pc, d_points, dc, rhoc, odf);
      dump(out, d_points);
      // CLUECUDAClusterizer::produce, then the CUDA CLUEOutputProducer's D2H
      PointsCloudCUDA d_cuda(n);
      if (!cuda_algo) cuda_algo = std::make_unique<CLUEAlgoGB300CUDA>(dc, rhoc, odf, stream);
      cuda_algo->makeClusters(pc, d_cuda, stream);
      PointsCloud results = pc;
      CLUEAlgoGB300CUDA::transferToHost(d_cuda, results, stream);
      dump(out, results);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  cudaStreamDestroy(stream);
  std::fclose(in);
  std::fclose(out);
  return 0;
}
