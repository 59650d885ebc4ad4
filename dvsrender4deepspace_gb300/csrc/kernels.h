// Device data views and kernel launchers of the GB300 DVS path.  Shared by
// kernels.cu (device code) and capi.cu (host orchestration).
#pragma once
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "dvs_internal.h"

namespace dvsgb {

struct SceneView {
  const BvhNode *nodes;       // reference geometry (FP32 child bounds)
  const BvhQNode *qnodes;     // FP16 child bounds (geometry bit 0), same indices
  int32_t geometry;           // bit 0: qnodes instead of nodes; bit 1: watertight test on vertex records
  const TriRecord *tris;
  const ShadeRecord *shade;
  const int32_t *pixel_of_rank;  // Morton rank -> row-major pixel index
  int32_t width, height, samples, has_albedo;
  float fx, fy, cx, cy;
  float coherent_span;  // largest origin spread a warp packet traverses as one interval bundle
  dvs_hapke hapke;
  int32_t rays;         // sub-rays a lane may carry: 1, 2 or 4 (used when samples^2 is a multiple)
  int32_t radiance_f32; // 1: the radiance chunk is written as float (read by an FP32 circuit), 0: as double
};

// Camera state at one circuit-cell midpoint, already interpolated
// (include/dvs/device_optics.cuh:13-26) with the light direction normalized.
struct alignas(16) CellPose {
  float px, py, pz, intensity;
  float qx, qy, qz, qw;
  float lx, ly, lz, pad;
};

// One circuit integration cell (event_sensor.cu:37-40): [t0, t1) of interval.
struct alignas(8) Cell {
  double t0, t1;
  int32_t interval;
  float dt;  // (float)(t1 - t0), rounded once on the host: the FP32 circuit's cell length
};

struct PixelParams {
  double threshold_pos, threshold_neg, charge_scale, refractory_time, reference_leak, reset_noise_std;
};
struct PhotoParams {
  double electrons_per_radiance, dark_electrons, integration_step;
  int32_t shot_noise;
  int32_t fp32_circuit;  // receptor/contrast arithmetic in FP32 (times and crossing solves stay FP64)
  int32_t philox;        // counter-based Philox noise keyed by (seed, pixel, cell index) instead of XORWOW
  uint32_t seed;
  int32_t chunk_f32;     // the circuit reads a float radiance chunk (FP32 circuits: the values it uses are floats)
};

// Pixel-circuit state, structure of arrays indexed by Morton rank.
struct CircuitState {
  double *receptor_log, *reference_log, *refractory_until, *threshold_pos, *threshold_neg;
  int8_t *reset_pending;
  curandStateXORWOW_t *rng;
  const int32_t *pixel;  // rank -> row-major pixel of the full image (the noise streams' key)
};

// Generated event before readout, aligned for device stores.
struct alignas(8) DevEvent {
  double t;
  float depth;
  int32_t rank;
  int16_t x, y;
  int8_t polarity;
  int8_t pad[3];
};

// Device readout (readout.cu).  Sort buffers for up to max_batch events:
// keys (order-preserving bits of t, then y<<16|x) and source indices, double
// buffered; which buffer holds the current order follows from `varying` (the
// radix passes whose digit differs between events move the keys, the others
// do nothing).
struct ReadoutSort {
  unsigned long long *kt[2];
  unsigned *kyx[2];
  unsigned *idx[2];
  unsigned long long *varying;  // [0]: OR over the batch of (time key ^ the first event's), [1]: the same for
                                // (y, x), [2]: the first event's time key
  unsigned *hist;               // per pass: counts per digit and sort block (digit-major, 256 x grid), scanned in place
  unsigned *digit_total;        // per pass: keys per digit (256)
};
// FIFO state and scratch.  ring: pending delivered events, ring_size a power
// of two; head/tail: monotone positions of the pending entries; plan: the
// release counts of the parallel path (-1: the serial path finished the batch).
struct ReadoutFifo {
  DevEvent *ring;
  unsigned long long ring_size, capacity;
  unsigned long long *head, *tail, *peak, *peak_batch, *dropped;
  double *available;
  double step, latency;  // 1 / bandwidth (0: no FIFO delay), latency
  unsigned long long *block_max;  // per sort block: the order-preserving key of max_k (t_k - k/B)
  double *completion, *delivery;
  int32_t *overflow, *status, *out_count;
  long long *plan;
  DevEvent *out;         // released events of the last submit or drain
  const int32_t *gate;   // optional: a nonzero word (the batch's error word) leaves the FIFO untouched
};
// Orders a batch of *count events by (t, y, x) and passes it through the
// FIFO at time *now (device memory, so a captured graph reads each step's);
// the released events land in f.out (*f.out_count of them).  grid: blocks
// of the sort and scan kernels (the sort's hist holds 256 x grid).
cudaError_t launch_readout_submit(const DevEvent *events, const int32_t *count, ReadoutSort s, ReadoutFifo f,
                                  const double *now, int grid, cudaStream_t st);
cudaError_t launch_readout_drain(ReadoutFifo f, int grid, cudaStream_t st);
// Kernels one launch_readout_submit enqueues (delayed: a bandwidth > 0 FIFO).
int readout_submit_launches(bool delayed);

// Error word bits (host maps them to DVS_ERR_* with capacity first, as
// event_sensor.cu:300-301 tests code 1 before any other code).
enum : int32_t { kErrCapacity = 1, kErrOptical = 2, kErrStalled = 4 };

// Device counters.
enum : int { kCntPrimary = 0, kCntShadow = 1, kCntCells = 2, kCntSlots = 4 };

// Radiance knot of the adaptive path (optical_sampler.hpp:278): fraction of
// the window (negative: the segment ending here is traced exactly per cell).
struct OpticalKnot {
  double fraction, radiance;
};
// Refinement counters (OpticalRefinementStats, optical_sampler.hpp:281).
enum : int { kRefTraced = 0, kRefFallback = 1, kRefMaxKnots = 2, kRefExactSegments = 3, kRefSlots = 4 };

// ---- launchers (return cudaGetLastError()) ----------------------------------
cudaError_t launch_pose_from_state(const dvs_optical_state *state, CellPose *out, cudaStream_t s);
cudaError_t launch_poses_from_states(const dvs_optical_state *states, int n, CellPose *out, cudaStream_t s);
// Motion-blur exposure: image[pixel] = sum_j float(radiance[j][rank]) * weights[j], in pose order.
cudaError_t launch_blur_accumulate(int n_pix, int n_poses, const int32_t *pixel_of_rank, const double *radiance,
                                   const float *weights, float *image, cudaStream_t s);
cudaError_t launch_cell_poses(const dvs_optical_interval *ivs, const Cell *cells, int n_cells, CellPose *out,
                              cudaStream_t s);
// Radiance (and optionally depth) of every pixel at every cell in [c0, c0+nc).
// Output index: cell * n_pix + rank.  Invalid samples store NaN radiance.
// ---- multi-sensor batch (batch.cu) ----------------------------------------
// One sensor's share of a batch step's trace: its cells [c0, c0 + nc) traced
// into its radiance chunk.  first_item: the first work item (warp packet) of
// this sensor in the batch's item space; items are job-major.
constexpr int kMaxBatchJobs = 128;
struct TraceJob {
  SceneView view;
  const CellPose *poses;
  double *radiance;
  unsigned long long *counters;
  long long first_item;
  int32_t n_pix, c0, nc, cw_log2;
};
// A trace launch's whole job table, passed as the kernel's parameter block
// (22.5 KB at 128 jobs, within the 32 KB parameter limit).
struct TraceJobs {
  TraceJob jobs[kMaxBatchJobs];
  long long total_items;
  unsigned long long *next_item;  // work counter, zeroed before the launch
  int32_t n_jobs, pad;
};
// One sensor's share of a batch step's circuit launch; first_block: its first
// 128-thread block (blocks never straddle two sensors).
struct CircuitJob {
  PixelParams p;
  PhotoParams photo;
  CircuitState st;
  const Cell *cells;
  const double *radiance;
  int32_t *ev_count;
  double *slab_t;
  int8_t *slab_p;
  int32_t *error;
  unsigned long long *counters;
  int32_t n, c0, nc, max_events, first_block, pad;
};
// Work items of one sensor's trace share (warp packets of cw_log2 cells).
long long trace_job_items(int n_pix, int nc, int cw_log2);
// Persistent trace of every job's items: a grid of resident blocks whose warps
// pull items from jobs.next_item (zeroed by the caller on the same stream).
// rays: 1 or 2 sub-rays per lane for every job; geometry: the jobs' shared
// SceneView::geometry.
cudaError_t launch_trace_jobs(const TraceJobs &jobs, int rays, int geometry, cudaStream_t s);
// One circuit launch over every job's pixels (total_blocks blocks of 128).
cudaError_t launch_circuit_jobs(const CircuitJob *jobs, int n_jobs, int total_blocks, bool fp32, bool philox,
                                cudaStream_t s);

cudaError_t launch_trace_cells(const SceneView &scene, int n_pix, const CellPose *poses, int c0, int nc,
                               int cw_log2, double *radiance, float *depth, unsigned long long *counters,
                               cudaStream_t s);
cudaError_t launch_init_pixels(int n_pix, const int32_t *pixel_of_rank, const double *radiance, PixelParams p,
                               PhotoParams photo, double threshold_std, double threshold_min, unsigned seed,
                               CircuitState st, int32_t *error, cudaStream_t s);
cudaError_t launch_circuit(int n_pix, const Cell *cells, int c0, int nc, const double *radiance, PixelParams p,
                           PhotoParams photo, int max_events, CircuitState st, int32_t *ev_count, double *slab_t,
                           int8_t *slab_p, int32_t *error, unsigned long long *counters, cudaStream_t s);
cudaError_t launch_emit_events(int n_pix, const int32_t *pixel_of_rank, int width, int max_events,
                               const int32_t *ev_count, const double *slab_t, const int8_t *slab_p, DevEvent *out,
                               int32_t *out_count, cudaStream_t s);
cudaError_t launch_event_depth(const SceneView &scene, const dvs_optical_interval *ivs, int n_ivs, DevEvent *events,
                               const int32_t *count, int32_t *error, unsigned long long *counters,
                               cudaStream_t s);
// Same kernels over a list of Morton ranks (row r of the radiance chunk is rank rank_list[r]).
cudaError_t launch_trace_list(const SceneView &scene, int n_pix, const int32_t *rank_list, const CellPose *poses,
                              int c0, int nc, int cw_log2, double *radiance, float *depth, unsigned long long *counters,
                              cudaStream_t s);
cudaError_t launch_circuit_list(int n, const int32_t *rank_list, const Cell *cells, int c0, int nc,
                                const double *radiance, PixelParams p, PhotoParams photo, int max_events,
                                CircuitState st, int32_t *ev_count, double *slab_t, int8_t *slab_p, int32_t *error,
                                unsigned long long *counters, cudaStream_t s);
// Adaptive optical refinement (adaptive.cu).
// probe_poses: 5 poses of scratch; probe_radiance: 5 x n doubles of scratch.
cudaError_t launch_refine(const SceneView &scene, int n, const dvs_optical_interval *ivs, int n_ivs, double start,
                          double end, PhotoParams photo, double tolerance, CircuitState st, double charge,
                          int capacity, CellPose *probe_poses, double *probe_radiance, OpticalKnot *knots,
                          int32_t *counts, unsigned long long *ref_stats, int32_t *error,
                          unsigned long long *counters, cudaStream_t s);
cudaError_t launch_identify_exact(int n, const Cell *cells, int n_cells, double start, double end,
                                  const OpticalKnot *knots, int32_t *knot_counts, int capacity, int32_t *exact_cells,
                                  int32_t *exact_counts, int32_t *queue, int32_t *total,
                                  unsigned long long *ref_stats, cudaStream_t s);
cudaError_t launch_sample_exact(const SceneView &scene, const CellPose *poses, const int32_t *exact_cells,
                                const int32_t *queue, const int32_t *total, int capacity, double *exact_radiance,
                                int32_t *error, unsigned long long *counters, cudaStream_t s);
cudaError_t launch_integrate_knots(int n, const Cell *cells, int n_cells, double start, double end,
                                   const OpticalKnot *knots, const int32_t *knot_counts, int capacity,
                                   const int32_t *exact_cells, const double *exact_radiance,
                                   const int32_t *exact_counts, PixelParams p, PhotoParams photo, int max_events,
                                   CircuitState st, int32_t *ev_count, double *slab_t, int8_t *slab_p,
                                   int32_t *error, cudaStream_t s);
cudaError_t launch_compact_fallback(int n, const int32_t *knot_counts, int32_t *list, int32_t *total,
                                    cudaStream_t s);
cudaError_t launch_capture_probes(int n_probes, const int32_t *probe_ranks, const double *receptor_log,
                                  double *probe_state, cudaStream_t s);
cudaError_t launch_advance_probes(int n_probes, const int32_t *probe_ranks, const Cell *cells, int c0, int nc,
                                  const double *light, const OpticalKnot *knots, const int32_t *knot_counts,
                                  int capacity, double start, double end, PhotoParams photo, double charge,
                                  double *probe_state, cudaStream_t s);
// n photon counts of mean lambda: generator 0 = XORWOW (curand_init(seed, i, 0),
// poisson_electrons), 1 = Philox of pixel i at cell start cell_t0.
cudaError_t launch_poisson_draws(int generator, double lambda, unsigned seed, int n, double cell_t0, double *out,
                                 cudaStream_t s);
// Loads (without launching) every kernel a one-pose camera render of a scene
// with this geometry may launch: the kernels of launch_trace_cells with one
// cell and launch_radiance_to_float.
cudaError_t preload_camera_kernels(int geometry);
cudaError_t launch_radiance_to_float(int n_pix, const int32_t *pixel_of_rank, const double *radiance,
                                     const float *depth, float *image, float *depth_image, cudaStream_t s);

}  // namespace dvsgb
