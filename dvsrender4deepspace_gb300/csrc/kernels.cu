// Device code of the GB300 DVS hot path (sm_103a).
//
// Built with -fmad=false: every floating-point expression rounds exactly as
// the reference writes it (and as the oracle computes it on the CPU), so the
// ray directions, Moller-Trumbore results, shadow origins and the FP64
// circuit differ from the reference only where CUDA's transcendental
// functions differ from the host C library.
//
// Work decomposition
//   * trace_cells: one warp traces a packet of 32 (pixel, cell) samples --
//     32/CW Morton-adjacent pixels x CW consecutive circuit cells.  All lanes
//     walk the 8-wide BVH together (warp-uniform control flow); coherent
//     packets test one child per lane against the packet's ray intervals,
//     leaves are tested per lane, and each lane keeps its own closest hit.
//     The traversal stack is warp-uniform and lives in shared memory.
//   * circuit: one thread per pixel streams the per-cell radiance of a chunk
//     and integrates the pixel circuit in FP64 (pixel_model.hpp semantics).
//   * emit_events: warp prefix-sum compaction of the per-pixel event slabs.
//   * event_depth: depth re-trace at each event time (event_sensor.cu:51-59).
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "kernels.h"
#include "device_optics.cuh"
#include "device_circuit.cuh"
#include "trace_item.cuh"

namespace dvsgb {
namespace {

// ---- kernels ------------------------------------------------------------------------
__global__ void pose_from_state_kernel(const dvs_optical_state *state, CellPose *out) {
  // A pose used as given (initialize_pixels, event_sensor.cu:22): the
  // quaternion is not renormalized; only the light is normalized.
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const dvs_optical_state s = *state;
  const float3 ln = normalize(ld3(s.light));
  CellPose o;
  o.px = s.position.x; o.py = s.position.y; o.pz = s.position.z; o.intensity = s.intensity;
  o.qx = s.rotation.x; o.qy = s.rotation.y; o.qz = s.rotation.z; o.qw = s.rotation.w;
  o.lx = ln.x; o.ly = ln.y; o.lz = ln.z; o.pad = 0;
  *out = o;
}

__global__ void poses_from_states_kernel(const dvs_optical_state *states, int n, CellPose *out) {
  // pose_from_state_kernel for n states: pose as given, light normalized
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const dvs_optical_state s = states[i];
  const float3 ln = normalize(ld3(s.light));
  CellPose o;
  o.px = s.position.x; o.py = s.position.y; o.pz = s.position.z; o.intensity = s.intensity;
  o.qx = s.rotation.x; o.qy = s.rotation.y; o.qz = s.rotation.z; o.qw = s.rotation.w;
  o.lx = ln.x; o.ly = ln.y; o.lz = ln.z; o.pad = 0;
  out[i] = o;
}

__global__ void cell_poses_kernel(const dvs_optical_interval *ivs, const Cell *cells, int n, CellPose *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const Cell cell = cells[c];
  out[c] = pose_at(ivs[cell.interval], (cell.t0 + cell.t1) * .5);
}


template <int kMode, int kRays, int kGeo>
__global__ void __launch_bounds__(128, kRays == 4   ? DVS_TRACE_QUAD_MIN_BLOCKS
                                       : kRays == 2 ? DVS_TRACE_PAIR_MIN_BLOCKS
                                                    : DVS_TRACE_MIN_BLOCKS)
    trace_cells_kernel(SceneView S, int n_pix, const int32_t *rank_list, const CellPose *poses, int c0, int nc,
                       int cw_log2, double *radiance, float *depth_out, unsigned long long *counters) {
  __shared__ int s_code[kWarpsPerBlock][kStackSlots];
  __shared__ float s_t[kWarpsPerBlock][kStackSlots];
  __shared__ SubraySample s_subrays[kWarpsPerBlock][kSubrayTable];
  const int wib = threadIdx.x >> 5;
  const long long warp = (long long)(blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  trace_cells_item<kMode, kRays, kGeo>(S, n_pix, rank_list, poses, c0, nc, cw_log2, radiance, depth_out, counters,
                                       warp, s_code[wib], s_t[wib], s_subrays[wib]);
}

// Few poses per pixel: one warp per (pixel, pose), lanes carrying the
// pixel's sub-rays (sample_pixel_subrays).  Item w = (rank, cell) with
// consecutive warps on the same pixel.
template <int kMode, int kGeo>
__global__ void __launch_bounds__(128, DVS_TRACE_PAIR_MIN_BLOCKS)
    trace_subray_kernel(SceneView S, int n_pix, const int32_t *rank_list, const CellPose *poses, int c0, int nc,
                        double *radiance, float *depth_out, unsigned long long *counters) {
  __shared__ int s_code[kWarpsPerBlock][kStackSlots];
  __shared__ float s_t[kWarpsPerBlock][kStackSlots];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)(blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= (long long)n_pix * nc) return;  // warp-uniform
  const int rank = (int)(warp / nc), cell = (int)(warp % nc);
  const int pixel = __ldg(S.pixel_of_rank + (rank_list ? rank_list[rank] : rank));
  const CellPose pose = poses[c0 + cell];
  const PixelSample s = sample_pixel_subrays<kMode, kGeo>(S, pixel, pose, s_code[wib], s_t[wib]);
  if (lane == 0) {
    const size_t o = (size_t)cell * n_pix + rank;
    store_radiance(S, radiance, o, s.valid ? s.radiance : __longlong_as_double(0x7ff8000000000000ll));
    if (depth_out) depth_out[o] = s.depth;
    if (counters) {
      atomicAdd(counters + kCntPrimary, (unsigned long long)s.primary);
      atomicAdd(counters + kCntShadow, (unsigned long long)s.shadow);
    }
  }
}

template <class Rng>
__global__ void init_pixels_kernel(int n, const int32_t *pixel_of_rank, const double *radiance, PixelParams p,
                                   PhotoParams photo, double stddev, double minimum, unsigned seed, CircuitState st,
                                   int32_t *error) {
  // initialize_pixels (event_sensor.cu:18-28); Rng = XORWOW (the reference's
  // generator) or, in precision mode, the head of the pixel's Philox stream
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int pixel = pixel_of_rank[k];
  Rng rng;
  curand_init(seed, pixel, 0, &rng);
  const double rad = radiance[k];
  if (!isfinite(rad)) {
    atomicOr(error, kErrOptical);
    if constexpr (std::is_same<Rng, curandStateXORWOW_t>::value) st.rng[k] = rng;
    return;
  }
  const double u = log(fmax(1e-30, rad * photo.electrons_per_radiance + photo.dark_electrons));
  st.receptor_log[k] = u;
  st.reference_log[k] = u;
  st.refractory_until[k] = -1;
  st.threshold_pos[k] = fmax(minimum, p.threshold_pos + stddev * curand_normal_double(&rng));
  st.threshold_neg[k] = fmax(minimum, p.threshold_neg + stddev * curand_normal_double(&rng));
  st.reset_pending[k] = 0;
  if constexpr (std::is_same<Rng, curandStateXORWOW_t>::value) st.rng[k] = rng;
}

template <bool kF32, bool kPhilox>
__global__ void __launch_bounds__(128) circuit_kernel(int n, const int32_t *rank_list, const Cell *cells, int c0,
                                                      int nc, const double *radiance, PixelParams p,
                                                      PhotoParams photo, int max_events, CircuitState st,
                                                      int32_t *ev_count, double *slab_t, int8_t *slab_p,
                                                      int32_t *error, unsigned long long *counters) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  circuit_rank<kF32, kPhilox>(r, n, rank_list, cells, c0, nc, radiance, p, photo, max_events, st, ev_count, slab_t,
                              slab_p, error, counters);
}

__global__ void emit_events_kernel(int n, const int32_t *pixel_of_rank, int width, int max_events,
                                   const int32_t *ev_count, const double *slab_t, const int8_t *slab_p,
                                   DevEvent *out, int32_t *out_count) {
  // warp ballot/prefix-sum compaction; one atomic per warp
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int cnt = (k < n && ev_count[k] > 0) ? ev_count[k] : 0;
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int v = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) incl += v;
  }
  const int total = __shfl_sync(kFull, incl, 31);
  int base = 0;
  if (lane == 31 && total) base = atomicAdd(out_count, total);
  base = __shfl_sync(kFull, base, 31);
  if (!cnt) return;
  const int pixel = pixel_of_rank[k];
  const int16_t x = (int16_t)(pixel % width), y = (int16_t)(pixel / width);
  int o = base + incl - cnt;
  for (int j = 0; j < cnt; ++j, ++o) {
    DevEvent e;
    e.t = slab_t[(size_t)k * max_events + j];
    e.depth = -1.0f;
    e.rank = k;
    e.x = x;
    e.y = y;
    e.polarity = slab_p[(size_t)k * max_events + j];
    e.pad[0] = e.pad[1] = e.pad[2] = 0;
    out[o] = e;
  }
}

template <int kGeo>
__global__ void __launch_bounds__(128) event_depth_kernel(SceneView S, const dvs_optical_interval *ivs, int n_ivs,
                                                          DevEvent *events, const int32_t *count, int32_t *error,
                                                          unsigned long long *counters) {
  // event-time depth re-trace (event_sensor.cu:51-59); grid-stride over the
  // device-side event count, warps stay converged for the packet traversal.
  __shared__ int s_code[kWarpsPerBlock][kStackSlots];
  __shared__ float s_t[kWarpsPerBlock][kStackSlots];
  const int wib = threadIdx.x >> 5;
  const int n = *count;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
    const int e = base + lane;
    const bool active = e < n;
    DevEvent ev = active ? events[e] : DevEvent{};
    // first interval whose t1 >= t (the reference's forward scan, :54)
    int lo = 0, hi = n_ivs - 1;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (ev.t > ivs[mid].t1) lo = mid + 1; else hi = mid;
    }
    const CellPose pose = pose_at(ivs[lo], ev.t);
    const int pixel = active ? S.pixel_of_rank[ev.rank] : 0;
    const PixelSample s = sample_pixel_packet<kDepthOnly, kGeo>(S, pixel, active, pose, s_code[wib], s_t[wib], nullptr);
    if (active) {
      if (!s.valid) atomicOr(error, kErrOptical);
      events[e].depth = s.depth;
    }
    const unsigned prim = warp_sum(s.primary);
    if (lane == 0 && counters) atomicAdd(counters + kCntPrimary, (unsigned long long)prim);
  }
}

__global__ void radiance_to_float_kernel(int n, const int32_t *pixel_of_rank, const double *radiance,
                                         const float *depth, float *image, float *depth_image) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int pixel = pixel_of_rank[k];
  image[pixel] = (float)radiance[k];
  if (depth_image) depth_image[pixel] = depth[k];
}

// Time-weighted exposure of a motion-blur frame (apps/main_cam_blur.cpp:66-73):
// per pixel, in pose order, acc += float(radiance of pose j) * weight[j].
__global__ void blur_accumulate_kernel(int n, int n_poses, const int32_t *pixel_of_rank, const double *radiance,
                                       const float *weights, float *image) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float acc = 0.0f;
  for (int j = 0; j < n_poses; ++j) acc = acc + (float)radiance[(size_t)j * n + k] * __ldg(weights + j);
  image[pixel_of_rank[k]] = acc;
}

// Photon counts as the circuit kernels draw them, one per thread: generator 0
// is the reference's stream -- curand_init(seed, i, 0) and poisson_electrons,
// as the counts kernel of tests/test_sensor.cu:17-20 -- and generator 1 the
// precision mode's Philox stream of pixel i at the cell starting at cell_t0.
__global__ void poisson_draws_kernel(int generator, double lambda, unsigned seed, int n, double cell_t0,
                                     double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (generator == 0) {
    curandStateXORWOW_t rng;
    curand_init(seed, i, 0, &rng);
    out[i] = poisson_electrons(rng, lambda);
  } else {
    curandStatePhilox4_32_10_t ph = philox_at(seed, i, cell_t0);
    out[i] = poisson_electrons_philox(ph, (float)lambda);
  }
}

inline int blocks(long long threads, int per_block) { return (int)((threads + per_block - 1) / per_block); }

}  // namespace

cudaError_t launch_poisson_draws(int generator, double lambda, unsigned seed, int n, double cell_t0, double *out,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  poisson_draws_kernel<<<blocks(n, 128), 128, 0, s>>>(generator, lambda, seed, n, cell_t0, out);
  return cudaGetLastError();
}

// ---- launchers ----------------------------------------------------------------------
cudaError_t launch_pose_from_state(const dvs_optical_state *state, CellPose *out, cudaStream_t s) {
  pose_from_state_kernel<<<1, 32, 0, s>>>(state, out);
  return cudaGetLastError();
}

cudaError_t launch_poses_from_states(const dvs_optical_state *states, int n, CellPose *out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  poses_from_states_kernel<<<blocks(n, 128), 128, 0, s>>>(states, n, out);
  return cudaGetLastError();
}

cudaError_t launch_blur_accumulate(int n, int n_poses, const int32_t *pixel_of_rank, const double *radiance,
                                   const float *weights, float *image, cudaStream_t s) {
  blur_accumulate_kernel<<<blocks(n, 128), 128, 0, s>>>(n, n_poses, pixel_of_rank, radiance, weights, image);
  return cudaGetLastError();
}

cudaError_t launch_cell_poses(const dvs_optical_interval *ivs, const Cell *cells, int n, CellPose *out,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  cell_poses_kernel<<<blocks(n, 128), 128, 0, s>>>(ivs, cells, n, out);
  return cudaGetLastError();
}

namespace {
template <int kGeo>
void trace_list_geo(const SceneView &scene, int n_pix, const int32_t *rank_list, const CellPose *poses, int c0, int nc,
                    int cw_log2, double *radiance, float *depth, unsigned long long *counters, cudaStream_t s) {
  if (scene.samples * scene.samples >= 32 && nc <= 8) {
    // few poses per pixel: sub-ray packets (one warp per pixel and pose)
    const int grid = blocks((long long)n_pix * nc * 32, 128);
    if (depth)
      trace_subray_kernel<kRadianceDepth, kGeo><<<grid, 128, 0, s>>>(scene, n_pix, rank_list, poses, c0, nc, radiance,
                                                                     depth, counters);
    else
      trace_subray_kernel<kRadiance, kGeo><<<grid, 128, 0, s>>>(scene, n_pix, rank_list, poses, c0, nc, radiance,
                                                                nullptr, counters);
    return;
  }
  const int cw = 1 << cw_log2, ppw = 32 >> cw_log2;
  const long long warps = (long long)((n_pix + ppw - 1) / ppw) * ((nc + cw - 1) / cw);
  const int ss2 = scene.samples * scene.samples;
  // four rays per lane only in the reference format (the others keep two)
  const int rays = (kGeo == kGeoReference && scene.rays >= 4 && ss2 % 4 == 0) ? 4
                   : (scene.rays >= 2 && ss2 % 2 == 0)                       ? 2
                                                                              : 1;
  const int grid = blocks(warps * 32, 128);
#define DVS_TRACE_LAUNCH(MODE, RAYS, DEPTH)                                                                         \
  trace_cells_kernel<MODE, RAYS, kGeo><<<grid, 128, 0, s>>>(scene, n_pix, rank_list, poses, c0, nc, cw_log2,       \
                                                            radiance, DEPTH, counters)
  if (depth) {
    if constexpr (kGeo == kGeoReference)
      if (rays == 4) { DVS_TRACE_LAUNCH(kRadianceDepth, 4, depth); return; }
    if (rays == 2) DVS_TRACE_LAUNCH(kRadianceDepth, 2, depth);
    else DVS_TRACE_LAUNCH(kRadianceDepth, 1, depth);
  } else {
    if constexpr (kGeo == kGeoReference)
      if (rays == 4) { DVS_TRACE_LAUNCH(kRadiance, 4, nullptr); return; }
    if (rays == 2) DVS_TRACE_LAUNCH(kRadiance, 2, nullptr);
    else DVS_TRACE_LAUNCH(kRadiance, 1, nullptr);
  }
#undef DVS_TRACE_LAUNCH
}
}  // namespace

cudaError_t launch_trace_list(const SceneView &scene, int n_pix, const int32_t *rank_list, const CellPose *poses,
                              int c0, int nc, int cw_log2, double *radiance, float *depth, unsigned long long *counters,
                              cudaStream_t s) {
  if (n_pix <= 0 || nc <= 0) return cudaSuccess;
  switch (scene.geometry) {
    case kGeoHalfBounds:
      trace_list_geo<kGeoHalfBounds>(scene, n_pix, rank_list, poses, c0, nc, cw_log2, radiance, depth, counters, s);
      break;
    case kGeoWatertight:
      trace_list_geo<kGeoWatertight>(scene, n_pix, rank_list, poses, c0, nc, cw_log2, radiance, depth, counters, s);
      break;
    case kGeoHalfBounds | kGeoWatertight:
      trace_list_geo<kGeoHalfBounds | kGeoWatertight>(scene, n_pix, rank_list, poses, c0, nc, cw_log2, radiance,
                                                      depth, counters, s);
      break;
    default:
      trace_list_geo<kGeoReference>(scene, n_pix, rank_list, poses, c0, nc, cw_log2, radiance, depth, counters, s);
  }
  return cudaGetLastError();
}

cudaError_t launch_trace_cells(const SceneView &scene, int n_pix, const CellPose *poses, int c0, int nc, int cw_log2,
                               double *radiance, float *depth, unsigned long long *counters, cudaStream_t s) {
  return launch_trace_list(scene, n_pix, nullptr, poses, c0, nc, cw_log2, radiance, depth, counters, s);
}

cudaError_t launch_init_pixels(int n, const int32_t *pixel_of_rank, const double *radiance, PixelParams p,
                               PhotoParams photo, double stddev, double minimum, unsigned seed, CircuitState st,
                               int32_t *error, cudaStream_t s) {
  if (photo.philox)
    init_pixels_kernel<curandStatePhilox4_32_10_t><<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, radiance, p, photo,
                                                                                stddev, minimum, seed, st, error);
  else
    init_pixels_kernel<curandStateXORWOW_t><<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, radiance, p, photo, stddev,
                                                                         minimum, seed, st, error);
  return cudaGetLastError();
}

cudaError_t launch_circuit_list(int n, const int32_t *rank_list, const Cell *cells, int c0, int nc,
                                const double *radiance, PixelParams p, PhotoParams photo, int max_events,
                                CircuitState st, int32_t *ev_count, double *slab_t, int8_t *slab_p, int32_t *error,
                                unsigned long long *counters, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (photo.fp32_circuit && photo.philox)
    circuit_kernel<true, true><<<blocks(n, 128), 128, 0, s>>>(n, rank_list, cells, c0, nc, radiance, p, photo,
                                                              max_events, st, ev_count, slab_t, slab_p, error, counters);
  else if (photo.fp32_circuit)
    circuit_kernel<true, false><<<blocks(n, 128), 128, 0, s>>>(n, rank_list, cells, c0, nc, radiance, p, photo,
                                                               max_events, st, ev_count, slab_t, slab_p, error, counters);
  else
    circuit_kernel<false, false><<<blocks(n, 128), 128, 0, s>>>(n, rank_list, cells, c0, nc, radiance, p, photo,
                                                                max_events, st, ev_count, slab_t, slab_p, error,
                                                                counters);
  return cudaGetLastError();
}

cudaError_t launch_circuit(int n, const Cell *cells, int c0, int nc, const double *radiance, PixelParams p,
                           PhotoParams photo, int max_events, CircuitState st, int32_t *ev_count, double *slab_t,
                           int8_t *slab_p, int32_t *error, unsigned long long *counters, cudaStream_t s) {
  return launch_circuit_list(n, nullptr, cells, c0, nc, radiance, p, photo, max_events, st, ev_count, slab_t, slab_p,
                             error, counters, s);
}

cudaError_t launch_emit_events(int n, const int32_t *pixel_of_rank, int width, int max_events, const int32_t *ev_count,
                               const double *slab_t, const int8_t *slab_p, DevEvent *out, int32_t *out_count,
                               cudaStream_t s) {
  emit_events_kernel<<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, width, max_events, ev_count, slab_t, slab_p,
                                                    out, out_count);
  return cudaGetLastError();
}

cudaError_t launch_event_depth(const SceneView &scene, const dvs_optical_interval *ivs, int n_ivs, DevEvent *events,
                               const int32_t *count, int32_t *error, unsigned long long *counters, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  switch (scene.geometry) {
    case kGeoHalfBounds:
      event_depth_kernel<kGeoHalfBounds><<<sms * 4, 128, 0, s>>>(scene, ivs, n_ivs, events, count, error, counters);
      break;
    case kGeoWatertight:
      event_depth_kernel<kGeoWatertight><<<sms * 4, 128, 0, s>>>(scene, ivs, n_ivs, events, count, error, counters);
      break;
    case kGeoHalfBounds | kGeoWatertight:
      event_depth_kernel<kGeoHalfBounds | kGeoWatertight><<<sms * 4, 128, 0, s>>>(scene, ivs, n_ivs, events, count,
                                                                                 error, counters);
      break;
    default:
      event_depth_kernel<kGeoReference><<<sms * 4, 128, 0, s>>>(scene, ivs, n_ivs, events, count, error, counters);
  }
  return cudaGetLastError();
}

namespace {
template <int kGeo>
cudaError_t preload_camera_geo() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, trace_subray_kernel<kRadianceDepth, kGeo>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_subray_kernel<kRadiance, kGeo>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadianceDepth, 1, kGeo>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadianceDepth, 2, kGeo>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadiance, 1, kGeo>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadiance, 2, kGeo>);
  if constexpr (kGeo == kGeoReference) {
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadianceDepth, 4, kGeo>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, trace_cells_kernel<kRadiance, 4, kGeo>);
  }
  return e;
}
}  // namespace

cudaError_t preload_camera_kernels(int geometry) {
  // cudaFuncGetAttributes loads a kernel that lazy module loading has not
  // loaded yet, so a later launch of it allocates nothing
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, radiance_to_float_kernel);
  if (e != cudaSuccess) return e;
  switch (geometry) {
    case kGeoHalfBounds: return preload_camera_geo<kGeoHalfBounds>();
    case kGeoWatertight: return preload_camera_geo<kGeoWatertight>();
    case kGeoHalfBounds | kGeoWatertight: return preload_camera_geo<kGeoHalfBounds | kGeoWatertight>();
    default: return preload_camera_geo<kGeoReference>();
  }
}

cudaError_t launch_radiance_to_float(int n, const int32_t *pixel_of_rank, const double *radiance, const float *depth,
                                     float *image, float *depth_image, cudaStream_t s) {
  radiance_to_float_kernel<<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, radiance, depth, image, depth_image);
  return cudaGetLastError();
}

}  // namespace dvsgb
