// Adaptive optical refinement on the GB300 path (replaces the reference's
// OpticalSampler::refine / prepare_exact_cells and EventSensor::
// process_adaptive kernels: src/cuda/optical_sampler.cu:25-138,
// src/cuda/event_sensor.cu:88-150).
//
// Per pixel, the radiance over a batch window is probed at 0, 1/4, 1/2, 3/4
// and 1 and bisected until a segment's linear interpolation predicts the
// receptor voltage within 1e-3 of the pixel's smaller threshold; segments
// that stay unresolved at the circuit-cell scale are marked for exact
// tracing of the cells inside them.  The circuit then integrates every
// native cell from the interpolated (or exactly traced) radiance.
//
// GB300 mapping: the reference gives each pixel a warp whose lanes split the
// sub-rays.  Here a lane owns a pixel and runs its own refinement stack; the
// 32 Morton-adjacent pixels of a warp probe in lock-step, so every probe is
// one coherent warp packet through the BVH (lanes with nothing to probe ride
// along inactive).  The probe value is the pixel's serial sub-ray mean, the
// same double the reference's warp_radiance returns.
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"
#include "device_optics.cuh"
#include "device_circuit.cuh"

namespace dvsgb {
namespace {

constexpr int kRefineStack = 16;  // optical_sampler.cu:43

struct RefineEntry {
  double a, b, left, middle, right;
};

// native_pose (optical_sampler.cu:26-30): the interval holding t.
__device__ __forceinline__ CellPose native_pose(const dvs_optical_interval *ivs, int count, double t) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int m = (lo + hi) / 2;
    if (t > ivs[m].t1) lo = m + 1; else hi = m;
  }
  return pose_at(ivs[lo], t);
}

// One lock-step probe: lanes with `want` trace their pixel at their time.
template <int kGeo>
__device__ __forceinline__ double probe(const SceneView &S, int pixel, bool want, const dvs_optical_interval *ivs,
                                        int n_ivs, double t, int *sc, float *stt, bool &bad, unsigned &rays) {
  const CellPose pose = native_pose(ivs, n_ivs, want ? t : ivs[0].t0);
  const PixelSample s = sample_pixel_packet<kRadiance, kGeo>(S, pixel, want, pose, sc, stt, nullptr);
  if (want && (!s.valid || !isfinite(s.radiance))) bad = true;
  rays += s.primary + s.shadow;
  return s.radiance;
}

__device__ __forceinline__ double segment_fraction(const OpticalKnot *values, int a) { return fabs(values[a].fraction); }

// The poses of the five initial probes (0, 1/4, 1/2, 3/4, 1 of the window).
__global__ void probe_poses_kernel(const dvs_optical_interval *ivs, int n_ivs, double start, double end,
                                   CellPose *out) {
  const int j = threadIdx.x;
  if (j < 5) out[j] = native_pose(ivs, n_ivs, start + (end - start) * j * .25);
}

// refine_pixels (optical_sampler.cu:39-84), one pixel per lane.  The five
// initial probes come traced by the native trace kernel (initial[j * n +
// rank]: every pixel is probed at the same five times, so they are five
// circuit cells of a temporal warp packet); the bisection probes, which only
// some pixels need, are traced here.
template <int kGeo>
__global__ void __launch_bounds__(128) refine_kernel(SceneView S, int n, const dvs_optical_interval *ivs, int n_ivs,
                                                     double start, double end, PhotoParams photo, double tolerance,
                                                     CircuitState st, double charge, int capacity,
                                                     const double *initial_radiance, OpticalKnot *knots,
                                                     int32_t *counts, unsigned long long *ref_stats,
                                                     int32_t *error, unsigned long long *counters) {
  __shared__ int s_code[4][kStackSlots];
  __shared__ float s_t[4][kStackSlots];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rank = blockIdx.x * blockDim.x + threadIdx.x;
  if (__all_sync(kFull, rank >= n)) return;  // warp-uniform
  const bool mine = rank < n;
  const int pixel = mine ? S.pixel_of_rank[rank] : 0;
  int *sc = s_code[wib];
  float *stt = s_t[wib];
  bool bad = false;
  unsigned rays = 0;
  double initial[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    initial[j] = mine ? initial_radiance[(size_t)j * n + rank] : 0.0;
    if (mine && !isfinite(initial[j])) bad = true;
  }
  RefineEntry stack[kRefineStack];
  int top = 0, written = 0;
  bool fallback = false;
  unsigned long long queries = 5;
  OpticalKnot *out = knots + (size_t)(mine ? rank : 0) * capacity;
  double v0 = 0, budget = 0;
  if (mine) {
    stack[0] = {.5, 1, initial[2], initial[3], initial[4]};
    stack[1] = {0, .5, initial[0], initial[1], initial[2]};
    top = 2;
    out[0] = {0, initial[0]};
    written = 1;
    v0 = st.receptor_log[rank];
    budget = 1e-3 * fmin(st.threshold_pos[rank], st.threshold_neg[rank]);  // kOpticalVoltageThresholdFraction
  }
  int exact_segments = 0;
  while (__any_sync(kFull, mine && top > 0 && !fallback)) {
    const bool work = mine && top > 0 && !fallback;
    bool need = false;
    double ta = 0, tb = 0, mid = 0;
    RefineEntry e{0, 0, 0, 0, 0};
    if (work) {
      e = stack[--top];
      const double actual = e.middle * photo.electrons_per_radiance + photo.dark_electrons;
      const double estimate = (e.left + e.right) * .5 * photo.electrons_per_radiance + photo.dark_electrons;
      const double residual = fabs(log(fmax(1e-30, actual) / fmax(1e-30, estimate)));
      const double leaf_duration = (e.b - e.a) * (end - start);
      const double voltage_error = fabs(receptor_log_at(v0, actual, leaf_duration, charge) -
                                        receptor_log_at(v0, estimate, leaf_duration, charge));
      if (voltage_error <= budget && (residual <= tolerance || fmax(actual, estimate) * leaf_duration < 1.0)) {
        if (written + 2 > capacity) {
          fallback = true;
        } else {
          out[written] = {(e.a + e.b) * .5, e.middle};
          out[written + 1] = {e.b, e.right};
          written += 2;
        }
      } else if ((e.b - e.a) * (end - start) <= photo.integration_step || top + 2 > kRefineStack) {
        // unresolved at the electrical sampling scale: exact tracing
        if (written >= capacity) {
          fallback = true;
        } else {
          out[written] = {-e.b, e.right};
          ++written;
          ++exact_segments;
        }
      } else {
        need = true;
        mid = (e.a + e.b) * .5;
        ta = start + (end - start) * (e.a + mid) * .5;
        tb = start + (end - start) * (mid + e.b) * .5;
      }
    }
    if (__any_sync(kFull, need)) {
      const double left_mid = probe<kGeo>(S, pixel, need, ivs, n_ivs, ta, sc, stt, bad, rays);
      const double right_mid = probe<kGeo>(S, pixel, need, ivs, n_ivs, tb, sc, stt, bad, rays);
      if (need) {
        queries += 2;
        stack[top] = {mid, e.b, e.middle, right_mid, e.right};
        stack[top + 1] = {e.a, mid, e.left, left_mid, e.middle};
        top += 2;
      }
    }
  }
  if (bad) atomicOr(error, kErrOptical);
  if (mine) {
    counts[rank] = fallback ? -1 : written;
    atomicAdd(ref_stats + kRefTraced, queries);
    if (fallback) atomicAdd(ref_stats + kRefFallback, 1ull);
    else atomicMax(ref_stats + kRefMaxKnots, (unsigned long long)written);
    if (exact_segments) atomicAdd(ref_stats + kRefExactSegments, (unsigned long long)exact_segments);
  }
  const unsigned wr = __reduce_add_sync(kFull, rays);
  if (lane == 0 && counters) atomicAdd(counters + kCntPrimary, (unsigned long long)wr);
}

// identify_exact_cells (optical_sampler.cu:114-131): cells whose midpoint falls
// in a marked segment are queued for exact tracing.
__global__ void identify_exact_kernel(int n, const Cell *cells, int n_cells, double start, double end,
                                      const OpticalKnot *knots, int32_t *knot_counts, int capacity,
                                      int32_t *exact_cells, int32_t *exact_counts, int32_t *queue, int32_t *total,
                                      unsigned long long *ref_stats) {
  const int rank = blockIdx.x * blockDim.x + threadIdx.x;
  if (rank >= n) return;
  exact_counts[rank] = 0;
  const int size = knot_counts[rank];
  if (size < 0) return;
  const OpticalKnot *values = knots + (size_t)rank * capacity;
  int a = 0, used = 0;
  for (int c = 0; c < n_cells; ++c) {
    const double fraction = ((cells[c].t0 + cells[c].t1) * .5 - start) / (end - start);
    while (a + 2 < size && fraction > fabs(values[a + 1].fraction)) ++a;
    if (values[a + 1].fraction < 0) {
      if (used == capacity) {
        knot_counts[rank] = -1;
        atomicAdd(ref_stats + kRefFallback, 1ull);
        return;
      }
      exact_cells[(size_t)rank * capacity + used++] = c;
    }
  }
  exact_counts[rank] = used;
  if (!used) return;
  const int offset = atomicAdd(total, used);
  for (int j = 0; j < used; ++j) queue[offset + j] = rank * capacity + j;
}

// sample_exact_queries (optical_sampler.cu:132-138): one queued cell per lane,
// grid-stride over the device-side queue length.
template <int kGeo>
__global__ void __launch_bounds__(128) sample_exact_kernel(SceneView S, const CellPose *poses,
                                                           const int32_t *exact_cells, const int32_t *queue,
                                                           const int32_t *total, int capacity, double *exact_radiance,
                                                           int32_t *error, unsigned long long *counters) {
  __shared__ int s_code[4][kStackSlots];
  __shared__ float s_t[4][kStackSlots];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int count = *total;
  const int stride = gridDim.x * blockDim.x;
  for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < count; base += stride) {
    const int q = base + lane;
    const bool active = q < count;
    const int slot = active ? queue[q] : 0;
    const int rank = slot / capacity;
    const int pixel = active ? S.pixel_of_rank[rank] : 0;
    const CellPose pose = poses[active ? exact_cells[slot] : 0];
    const PixelSample s = sample_pixel_packet<kRadiance, kGeo>(S, pixel, active, pose, s_code[wib], s_t[wib], nullptr);
    if (active) {
      if (!s.valid || !isfinite(s.radiance)) atomicOr(error, kErrOptical);
      exact_radiance[slot] = s.radiance;
    }
    const unsigned r = __reduce_add_sync(kFull, s.primary + s.shadow);
    if (lane == 0 && counters) atomicAdd(counters + kCntPrimary, (unsigned long long)r);
  }
}

// integrate_optical_knots (event_sensor.cu:88-114): every native cell from the
// knots (or its exactly traced radiance); events carry no depth.
__global__ void __launch_bounds__(128) integrate_knots_kernel(int n, const Cell *cells, int n_cells, double start,
                                                              double end, const OpticalKnot *knots,
                                                              const int32_t *knot_counts, int capacity,
                                                              const int32_t *exact_cells, const double *exact_radiance,
                                                              const int32_t *exact_counts, PixelParams p,
                                                              PhotoParams photo, int max_events, CircuitState st,
                                                              int32_t *ev_count, double *slab_t, int8_t *slab_p,
                                                              int32_t *error) {
  const int rank = blockIdx.x * blockDim.x + threadIdx.x;
  if (rank >= n || knot_counts[rank] < 0) return;
  const OpticalKnot *values = knots + (size_t)rank * capacity;
  const int size = knot_counts[rank];
  const int n_exact = exact_counts ? exact_counts[rank] : 0;
  const int32_t *my_exact = exact_cells + (size_t)rank * capacity;
  const double *my_exact_rad = exact_radiance + (size_t)rank * capacity;
  PixelRegs s{st.receptor_log[rank], st.reference_log[rank], st.refractory_until[rank], st.threshold_pos[rank],
              st.threshold_neg[rank], st.reset_pending[rank] != 0};
  curandStateXORWOW_t rng = st.rng[rank];
  double *my_t = slab_t + (size_t)rank * max_events;
  int8_t *my_p = slab_p + (size_t)rank * max_events;
  int a = 0, exact_index = 0, count = 0, failed = 0;
  for (int c = 0; c < n_cells; ++c) {
    const double t0 = cells[c].t0, t1 = cells[c].t1;
    const double fraction = ((t0 + t1) * .5 - start) / (end - start);
    while (a + 2 < size && fraction > segment_fraction(values, a + 1)) ++a;
    const double weight =
        (fraction - segment_fraction(values, a)) / (segment_fraction(values, a + 1) - segment_fraction(values, a));
    double light = values[a].radiance + (values[a + 1].radiance - values[a].radiance) * weight;
    if (exact_index < n_exact && my_exact[exact_index] == c) light = my_exact_rad[exact_index++];
    double rate = fmax(0.0, light) * photo.electrons_per_radiance + photo.dark_electrons;
    if (photo.shot_noise) rate = poisson_electrons(rng, rate * (t1 - t0)) / (t1 - t0);
    const int emitted = advance_pixel(s, p, rate, t0, t1, my_t + count, my_p + count, max_events - count, rng);
    if (emitted == -1) { failed = kErrCapacity; break; }
    if (emitted == -2) { failed = kErrStalled; break; }
    count += emitted;
  }
  st.receptor_log[rank] = s.receptor_log;
  st.reference_log[rank] = s.reference_log;
  st.refractory_until[rank] = s.refractory_until;
  st.reset_pending[rank] = s.reset_pending ? 1 : 0;
  st.rng[rank] = rng;
  if (failed) {
    atomicOr(error, failed);
    ev_count[rank] = -1;
  } else {
    ev_count[rank] = count;
  }
}

// compact_fallback (event_sensor.cu:116-118).
__global__ void compact_fallback_kernel(int n, const int32_t *knot_counts, int32_t *list, int32_t *total) {
  const int rank = blockIdx.x * blockDim.x + threadIdx.x;
  if (rank < n && knot_counts[rank] < 0) list[atomicAdd(total, 1)] = rank;
}

// advance_mean_probes (event_sensor.cu:138-150): receptor driven by exact and
// by knot-interpolated light for the probe pixels, over one cell chunk.
__global__ void advance_probes_kernel(int n_probes, const int32_t *probe_ranks, const Cell *cells, int c0, int nc,
                                      const double *light, const OpticalKnot *knots, const int32_t *knot_counts,
                                      int capacity, double start, double end, PhotoParams photo, double charge,
                                      double *probe_state) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_probes) return;
  const int rank = probe_ranks[i];
  const OpticalKnot *values = knots + (size_t)rank * capacity;
  double ex = probe_state[2 * i], ca = probe_state[2 * i + 1];
  for (int c = 0; c < nc; ++c) {
    const Cell cell = cells[c0 + c];
    const double exact = light[(size_t)c * n_probes + i];
    double cached = exact;
    if (knot_counts[rank] >= 0) {
      int a = 0;
      const double fraction = ((cell.t0 + cell.t1) * .5 - start) / (end - start);
      while (a + 2 < knot_counts[rank] && fraction > fabs(values[a + 1].fraction)) ++a;
      const double weight =
          (fraction - fabs(values[a].fraction)) / (fabs(values[a + 1].fraction) - fabs(values[a].fraction));
      if (values[a + 1].fraction >= 0) cached = values[a].radiance + (values[a + 1].radiance - values[a].radiance) * weight;
    }
    ex = receptor_log_at(ex, exact * photo.electrons_per_radiance + photo.dark_electrons, cell.t1 - cell.t0, charge);
    ca = receptor_log_at(ca, fmax(0.0, cached) * photo.electrons_per_radiance + photo.dark_electrons,
                         cell.t1 - cell.t0, charge);
  }
  probe_state[2 * i] = ex;
  probe_state[2 * i + 1] = ca;
}

__global__ void capture_probes_kernel(int n_probes, const int32_t *probe_ranks, const double *receptor_log,
                                      double *probe_state) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_probes) return;
  const double u = receptor_log[probe_ranks[i]];
  probe_state[2 * i] = u;
  probe_state[2 * i + 1] = u;
}

inline int blocks_of(long long threads, int per_block) { return (int)((threads + per_block - 1) / per_block); }
int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace

cudaError_t launch_refine(const SceneView &scene, int n, const dvs_optical_interval *ivs, int n_ivs, double start,
                          double end, PhotoParams photo, double tolerance, CircuitState st, double charge,
                          int capacity, CellPose *probe_poses, double *probe_radiance, OpticalKnot *knots,
                          int32_t *counts, unsigned long long *ref_stats, int32_t *error,
                          unsigned long long *counters, cudaStream_t s) {
  // the five initial probes of every pixel: five cells of the native trace
  // kernel (8 cells per warp packet: 4 pixels x 5 probe times)
  probe_poses_kernel<<<1, 32, 0, s>>>(ivs, n_ivs, start, end, probe_poses);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_trace_cells(scene, n, probe_poses, 0, 5, 3, probe_radiance, nullptr, counters, s);
  if (e != cudaSuccess) return e;
#define DVS_REFINE(G)                                                                                         \
  refine_kernel<G><<<blocks_of(n, 128), 128, 0, s>>>(scene, n, ivs, n_ivs, start, end, photo, tolerance, st, charge, \
                                                     capacity, probe_radiance, knots, counts, ref_stats, error,     \
                                                     counters)
  switch (scene.geometry) {
    case kGeoHalfBounds: DVS_REFINE(kGeoHalfBounds); break;
    case kGeoWatertight: DVS_REFINE(kGeoWatertight); break;
    case kGeoHalfBounds | kGeoWatertight: DVS_REFINE(kGeoHalfBounds | kGeoWatertight); break;
    default: DVS_REFINE(kGeoReference);
  }
#undef DVS_REFINE
  return cudaGetLastError();
}

cudaError_t launch_identify_exact(int n, const Cell *cells, int n_cells, double start, double end,
                                  const OpticalKnot *knots, int32_t *knot_counts, int capacity, int32_t *exact_cells,
                                  int32_t *exact_counts, int32_t *queue, int32_t *total,
                                  unsigned long long *ref_stats, cudaStream_t s) {
  identify_exact_kernel<<<blocks_of(n, 128), 128, 0, s>>>(n, cells, n_cells, start, end, knots, knot_counts, capacity,
                                                          exact_cells, exact_counts, queue, total, ref_stats);
  return cudaGetLastError();
}

cudaError_t launch_sample_exact(const SceneView &scene, const CellPose *poses, const int32_t *exact_cells,
                                const int32_t *queue, const int32_t *total, int capacity, double *exact_radiance,
                                int32_t *error, unsigned long long *counters, cudaStream_t s) {
#define DVS_EXACT(G)                                                                                       \
  sample_exact_kernel<G><<<sm_count() * 8, 128, 0, s>>>(scene, poses, exact_cells, queue, total, capacity,     \
                                                        exact_radiance, error, counters)
  switch (scene.geometry) {
    case kGeoHalfBounds: DVS_EXACT(kGeoHalfBounds); break;
    case kGeoWatertight: DVS_EXACT(kGeoWatertight); break;
    case kGeoHalfBounds | kGeoWatertight: DVS_EXACT(kGeoHalfBounds | kGeoWatertight); break;
    default: DVS_EXACT(kGeoReference);
  }
#undef DVS_EXACT
  return cudaGetLastError();
}

cudaError_t launch_integrate_knots(int n, const Cell *cells, int n_cells, double start, double end,
                                   const OpticalKnot *knots, const int32_t *knot_counts, int capacity,
                                   const int32_t *exact_cells, const double *exact_radiance,
                                   const int32_t *exact_counts, PixelParams p, PhotoParams photo, int max_events,
                                   CircuitState st, int32_t *ev_count, double *slab_t, int8_t *slab_p,
                                   int32_t *error, cudaStream_t s) {
  integrate_knots_kernel<<<blocks_of(n, 128), 128, 0, s>>>(n, cells, n_cells, start, end, knots, knot_counts,
                                                           capacity, exact_cells, exact_radiance, exact_counts, p,
                                                           photo, max_events, st, ev_count, slab_t, slab_p, error);
  return cudaGetLastError();
}

cudaError_t launch_compact_fallback(int n, const int32_t *knot_counts, int32_t *list, int32_t *total,
                                    cudaStream_t s) {
  compact_fallback_kernel<<<blocks_of(n, 128), 128, 0, s>>>(n, knot_counts, list, total);
  return cudaGetLastError();
}

cudaError_t launch_capture_probes(int n_probes, const int32_t *probe_ranks, const double *receptor_log,
                                  double *probe_state, cudaStream_t s) {
  capture_probes_kernel<<<blocks_of(n_probes, 128), 128, 0, s>>>(n_probes, probe_ranks, receptor_log, probe_state);
  return cudaGetLastError();
}

cudaError_t launch_advance_probes(int n_probes, const int32_t *probe_ranks, const Cell *cells, int c0, int nc,
                                  const double *light, const OpticalKnot *knots, const int32_t *knot_counts,
                                  int capacity, double start, double end, PhotoParams photo, double charge,
                                  double *probe_state, cudaStream_t s) {
  advance_probes_kernel<<<blocks_of(n_probes, 128), 128, 0, s>>>(n_probes, probe_ranks, cells, c0, nc, light, knots,
                                                                 knot_counts, capacity, start, end, photo, charge,
                                                                 probe_state);
  return cudaGetLastError();
}

}  // namespace dvsgb
