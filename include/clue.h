/*
 * clue.h -- C ABI of the GB300-native CLUE clustering path.
 *
 * Drop-in for the clusterizer producer of tonydp03/heterogeneous-clue:
 * PointsCloud in (float x, y, weight; int32 layer in [0, 100)), the
 * dc / rhoc / outlierDeltaFactor parameters in, and per point rho, delta,
 * nearestHigher, isSeed and clusterIndex out, bit-identical to the serial
 * backend.  Plain pointers and sizes only; no C++ or torch types.
 *
 * Threading: a handle is externally synchronised (one caller at a time);
 * distinct handles may run concurrently, each on its own CUDA stream.  The
 * serving entry points (clue_server_*) are thread-safe.
 *
 * Errors: every entry point returns a clue_status; clue_last_error() gives a
 * message for the calling thread.  Nothing aborts the process.
 */
#ifndef CLUE_GB300_CLUE_H
#define CLUE_GB300_CLUE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum clue_status {
  CLUE_OK = 0,
  CLUE_EINVAL = 1,   /* bad argument, n < 0, layer outside [0, n_layers) */
  CLUE_ENOMEM = 2,   /* the request needs more device memory than the budget */
  CLUE_ECUDA = 3,    /* a CUDA runtime call failed (no device, launch error) */
  CLUE_ETIMEOUT = 4, /* a bounded wait ran out */
  CLUE_EBUSY = 5     /* request not finished yet (clue_server_poll) */
} clue_status;

/* Memory-space and path flags of the run calls. */
#define CLUE_HOST_MEMORY 0   /* pointers are host memory; the call returns when outputs are written */
#define CLUE_DEVICE_MEMORY 1 /* pointers are device memory; work is queued on the handle's stream */
#define CLUE_PLAIN 2         /* run events one at a time (the per-event launch sequence) */
#define CLUE_NO_GRAPH 4      /* launch the batched pipeline directly instead of replaying a CUDA graph */
#define CLUE_NO_PIPELINE 8   /* host memory: one H2D, kernels, D2H sequence instead of overlapped sub-batches */

/* Parameters (src/serial/DataFormats/CLUE_config.h:8-13, without produceOutput). */
typedef struct clue_params {
  float dc;
  float rhoc;
  float outlierDeltaFactor;
} clue_params;

/* Caller-owned outputs, one entry per point, in input order
 * (the output half of PointsCloudSerial, src/serial/DataFormats/PointsCloud.h:33-38).
 * nearestHigher is an event-local index, or -1. */
typedef struct clue_outputs {
  float* rho;
  float* delta;
  int32_t* nearestHigher;
  int32_t* isSeed;
  int32_t* clusterIndex;
} clue_outputs;

/* Work decomposition of the batched kernels.  None of it changes results. */
typedef struct clue_tuning {
  int32_t threads;        /* threads per CTA of the layer kernel: 128, 256, 512 or 1024 */
  int32_t layer_capacity; /* points of one layer held on-chip; larger layers use HBM scratch */
  float work_tile_cm;     /* reserved, must be 0: the 5 cm tiles are the reference's and a layer is one work unit */
  int32_t ctas_per_sm;    /* 0 = as many as shared memory allows */
  int32_t big_threads;    /* second pass for layers above layer_capacity: threads per CTA, 0 = none */
  int32_t big_capacity;   /* on-chip points of that pass; larger layers use HBM scratch */
} clue_tuning;

typedef struct clue_handle clue_handle;

/* Replaces the CLUEAlgoSerial / CLUEAlgoCUDA constructors
 * (src/serial/plugin-CLUEClusterizer/CLUEAlgoSerial.h:9,
 *  src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.h:14-17).
 * device_budget_bytes caps the resident device memory (0 = 16 GiB).
 * cuda_stream is a cudaStream_t (NULL: the handle creates its own). */
int clue_create(const clue_params* params, size_t device_budget_bytes, int device, void* cuda_stream,
                clue_handle** out);
int clue_destroy(clue_handle* h);
int clue_set_params(clue_handle* h, const clue_params* params);

/* Moves later work of the handle to cuda_stream (NULL: back to a stream the
 * handle owns), after waiting for the handle's previous run.  Mirrors the
 * per-call stream argument of CLUEAlgoCUDA::makeClusters
 * (src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.h:21). */
int clue_set_stream(clue_handle* h, void* cuda_stream);

/* One event: replaces CLUEAlgoSerial::makeClusters
 * (src/serial/plugin-CLUEClusterizer/CLUEAlgoSerial.cc:18-35) and
 * CLUEAlgoCUDA::makeClusters (src/cuda/plugin-CLUEClusterizer/CLUEAlgoCUDA.cu:59-81). */
int clue_run_event(clue_handle* h, int32_t n, const float* x, const float* y, const int32_t* layer,
                   const float* weight, const clue_outputs* out, int flags);

/* n_events events concatenated in CSR order: event e is
 * [event_offsets[e], event_offsets[e+1]) of x, y, layer, weight and of the
 * outputs.  event_offsets is always HOST memory.  No reference counterpart:
 * it is the batched form of makeClusters over the reference's EDM streams
 * (src/serial/bin/StreamSchedule.cc:61-93). */
int clue_run_batch(clue_handle* h, int32_t n_events, const int64_t* event_offsets, const float* x, const float* y,
                   const int32_t* layer, const float* weight, const clue_outputs* out, int flags);

/* Waits for queued work (CLUE_DEVICE_MEMORY calls) and returns the first
 * error recorded on the device (e.g. a layer outside [0, 100)). */
int clue_synchronize(clue_handle* h);

/* What the last CLUE 2D run (clue_run_event / clue_run_batch) on a handle
 * queued: host<->device bytes (points, outputs, offset and chunk tables,
 * status words; device-memory runs copy only the tables and the status) and
 * kernel launches (a graph replay counts the kernels in the graph). */
typedef struct clue_run_stats {
  int64_t h2d_bytes;
  int64_t d2h_bytes;
  int64_t kernel_launches;
} clue_run_stats;
int clue_last_run_stats(clue_handle* h, clue_run_stats* stats);

/* Device bytes a batch of n_points points in n_events events needs. */
size_t clue_required_bytes(int32_t n_events, int64_t n_points, int flags);

/* Stages of the batched pipeline, in launch order. */
#define CLUE_N_STAGES 7 /* count, layer_scan (with the largest-first order when taken), scatter,
                           layers (which also counts seeds per chunk), seed_chunk_scan, seed_rank, label */

/* Runs one batch like clue_run_batch (device memory, direct launches) and
 * writes each stage's duration in milliseconds to stage_ms[CLUE_N_STAGES],
 * timed with CUDA events on the handle's stream.  The reference only times
 * whole runs (src/serial/bin/main.cc:194-238); this is the per-phase view. */
int clue_profile_batch(clue_handle* h, int32_t n_events, const int64_t* event_offsets, const float* x,
                       const float* y, const int32_t* layer, const float* weight, const clue_outputs* out,
                       float* stage_ms);

int clue_get_tuning(clue_handle* h, clue_tuning* t);
int clue_set_tuning(clue_handle* h, const clue_tuning* t);

/* Times the candidate work decompositions on this batch (device memory),
 * keeps the fastest in the handle, checks that every candidate gives
 * bit-identical outputs, and records the choice in cache_path (JSON lines,
 * keyed by GPU name and workload) when it is not NULL.  A cached choice is
 * reused without timing. */
int clue_autotune(clue_handle* h, int32_t n_events, const int64_t* event_offsets, const float* x, const float* y,
                  const int32_t* layer, const float* weight, const clue_outputs* out, const char* cache_path,
                  clue_tuning* chosen);

const char* clue_last_error(void);

/* One event through the batched kernels WITHOUT allocating anything: no
 * handle, no cudaMalloc/cudaFree, no allocating library call.  It has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory themselves (a host framework that pre-reserves the whole
 * device for its own pool, real-time or embedded code that must not touch
 * the allocator after start-up).  x, y, layer, weight and the outputs are
 * DEVICE pointers; work runs on cuda_stream (NULL = default stream) and the
 * call synchronises that stream before returning.
 * Scratch is one fixed 14 MB area compiled into the library (a static
 * __device__ array), so n is limited to 262,144 points; larger events get
 * CLUE_EINVAL.  The CUDA runtime creates that array, and loads the kernels'
 * code, lazily: on each device, the first call does it.  Make that first
 * call at start-up, before the framework reserves the device's memory for its
 * pool, and outside any stream capture: a call with n == 0 (every pointer
 * may then be NULL) does only this set-up.  The array stays until the
 * process exits.  All calls share the area: calls that overlap on the GPU
 * race; run them one at a time. */
int clue_run_event_noalloc(const clue_params* params, int32_t n, const float* x, const float* y,
                           const int32_t* layer, const float* weight, const clue_outputs* out, void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* CLUE3D (tracksterizer)                                                     */
/* ------------------------------------------------------------------------ */

/* Every default argument of the serial CLUE3D kernels
 * (src/serial/plugin-CLUETracksterizer/CLUE3DAlgoKernels.h:26-32,286-290,509-515)
 * and the layer count (ticl::TileConstants::nLayers,
 * src/serial/DataFormats/Common.h:14). */
typedef struct clue3d_params {
  int32_t n_layers;
  int32_t density_sibling_layers;
  float density_xy_distance_sqr;
  float kernel_density_factor;
  int32_t density_on_same_layer;
  int32_t nh_sibling_layers;
  int32_t nh_on_same_layer;
  float critical_xy_distance;
  float critical_z_distance_lyr;
  float critical_density;
  float critical_self_density;
  float outlier_multiplier;
} clue3d_params;

/* The reference defaults (94 layers, 3 sibling layers, 3.24 cm^2, 0.2, ...). */
void clue3d_default_params(clue3d_params* p);

/* Layer clusters (ClusterCollection, src/serial/DataFormats/ClusterCollection.h:6-19;
 * x and y are not read by the algorithm and are not passed). */
typedef struct clue3d_inputs {
  const float* z;
  const float* eta;
  const float* phi;
  const float* r_over_absz;
  const float* radius;
  const int32_t* layer;
  const float* energy;
  const int32_t* isSilicon;
} clue3d_inputs;

/* Outputs of ClusterCollectionSerial (ClusterCollection.h:35-40): delta is
 * (transverse distance, layer distance), nearestHigher is (layer, event-local
 * index); tracksterIndex is -1 for unassigned clusters. */
typedef struct clue3d_outputs {
  float* rho;
  float* delta_transverse;
  int32_t* delta_layers;
  int32_t* nh_layer;
  int32_t* nh_index;
  int32_t* isSeed;
  int32_t* tracksterIndex;
} clue3d_outputs;

/* Replaces CLUE3DAlgoSerial::makeTrackstersSoA
 * (src/serial/plugin-CLUETracksterizer/CLUE3DAlgoSerial.cc:42-50) over
 * n_events events in CSR order (event_offsets in HOST memory).
 * n_tracksters (host, may be NULL) receives the per-event trackster counts
 * (KernelFindAndAssignClustersSoA's return value) when the call is
 * synchronous (CLUE_HOST_MEMORY). */
int clue3d_run_batch(clue_handle* h, const clue3d_params* params, int32_t n_events, const int64_t* event_offsets,
                     const clue3d_inputs* in, const clue3d_outputs* out, int32_t* n_tracksters, int flags);

/* ------------------------------------------------------------------------ */
/* 2D -> 3D bridge: layer clusters of a clustered 2D batch, on the device.   */
/* No reference counterpart (the reference's CLUE3D reads raw3D files,       */
/* src/serial/bin/Source.cc:43-60).  Layer cluster c of event e is the set   */
/* of 2D points with clusterIndex c; energy = sum of weights (exact          */
/* fixed-point sums, so deterministic), x, y = weight-weighted means,        */
/* layer = the seed's, z = layer_z[layer], r_over_absz = r/|z|,              */
/* eta = asinh(z/r), phi = atan2(y, x).  Arrays are DEVICE memory;           */
/* event_offsets, cluster_offsets and layer_z are HOST memory.  Both calls   */
/* return when their work has finished.                                      */
/* ------------------------------------------------------------------------ */

typedef struct clue_bridge_params {
  int32_t n_layers;     /* entries of layer_z; a cluster's layer must be below it */
  const float* layer_z; /* z (cm) of each layer */
  float radius;         /* radius given to every layer cluster (cm) */
  int32_t isSilicon;    /* isSilicon given to every layer cluster */
} clue_bridge_params;

typedef struct clue_layer_clusters {
  float* x;
  float* y;
  float* z;
  float* eta;
  float* phi;
  float* r_over_absz;
  float* radius;
  int32_t* layer;
  float* energy;
  int32_t* isSilicon;
} clue_layer_clusters;

/* Layer clusters per event (the 2D seeds) as CSR offsets: cluster_offsets
 * (host, n_events + 1 entries) is written. */
int clue_bridge_count(clue_handle* h, int32_t n_events, const int64_t* event_offsets, const int32_t* isSeed,
                      int64_t* cluster_offsets);

/* Builds the layer clusters (out holds cluster_offsets[n_events] entries per
 * array, in event order, then cluster id order); the result is a CLUE3D
 * input for clue3d_run_batch with cluster_offsets as its event offsets. */
int clue_bridge_build(clue_handle* h, const clue_bridge_params* p, int32_t n_events, const int64_t* event_offsets,
                      const float* x, const float* y, const int32_t* layer, const float* weight,
                      const int32_t* isSeed, const int32_t* clusterIndex, const int64_t* cluster_offsets,
                      const clue_layer_clusters* out);

/* ------------------------------------------------------------------------ */
/* Serving: continuous batching of CLUE 2D events                            */
/* ------------------------------------------------------------------------ */

typedef struct clue_server clue_server;

typedef struct clue_server_config {
  size_t device_budget_bytes; /* total device memory for all in-flight batches (0 = 16 GiB) */
  int32_t max_inflight;       /* batches on the device at once, each on its own stream (>= 1) */
  int32_t max_batch_events;   /* events per batch at most */
  int32_t device;
} clue_server_config;

typedef struct clue_server_stats {
  int64_t completed;
  int64_t batches;
  double p50_ms;  /* latency from submit to outputs written, over completed requests */
  double p99_ms;
  double mean_batch_events;
  double max_inflight_seen;
  int64_t slot_capacity_points; /* largest event (points) admitted: it fits the budget while the other
                                   slots hold only their start-up buffers */
  int64_t memory_waits;         /* times the head of the queue waited for device memory to free up */
} clue_server_stats;

int clue_server_create(const clue_params* params, const clue_server_config* cfg, clue_server** out);
int clue_server_destroy(clue_server* s);

/* Queues one event (host pointers).  The inputs are copied before the call
 * returns; the output buffers must stay valid until the request completes.
 * Device memory is shared by the in-flight batches: each slot keeps buffers
 * for ordinary batches (sized at start within half of an equal share), and an
 * event larger than those takes, alone, what the others leave of the budget,
 * waiting for in-flight batches to finish when they hold it.  Returns
 * CLUE_ENOMEM only when the event could not fit even with every other slot
 * at its start-up buffers (slot_capacity_points). */
int clue_server_submit(clue_server* s, int32_t n, const float* x, const float* y, const int32_t* layer,
                       const float* weight, const clue_outputs* out, int64_t* request_id);

/* Queues n_events events at once (CSR event_offsets, host, over host x, y,
 * layer, weight; outs holds one clue_outputs per event; request_ids receives
 * n_events ids).  They enter the queue together, so they can share a batch.
 * Nothing is queued when an argument is rejected. */
int clue_server_submit_many(clue_server* s, int32_t n_events, const int64_t* event_offsets, const float* x,
                            const float* y, const int32_t* layer, const float* weight, const clue_outputs* outs,
                            int64_t* request_ids);

/* CLUE_OK when the request's outputs are written, CLUE_EBUSY while it is
 * pending (timeout_ms = 0), CLUE_ETIMEOUT when timeout_ms ran out; <0 waits
 * without limit.  latency_ms (may be NULL) receives submit-to-completion time. */
int clue_server_poll(clue_server* s, int64_t request_id, int32_t timeout_ms, double* latency_ms);

/* Blocks until every submitted request is complete (bounded by timeout_ms, <0 = no bound). */
int clue_server_drain(clue_server* s, int32_t timeout_ms);
int clue_server_get_stats(clue_server* s, clue_server_stats* st);
int clue_server_reset_stats(clue_server* s);

#ifdef __cplusplus
}
#endif

#endif /* CLUE_GB300_CLUE_H */
