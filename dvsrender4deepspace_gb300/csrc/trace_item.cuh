// Per-item device bodies of the trace and circuit launches, shared by the
// one-sensor kernels (kernels.cu) and the multi-sensor batch kernels
// (batch.cu).  Included after device_optics.cuh and device_circuit.cuh.
#pragma once
#include "device_circuit.cuh"
#include "device_optics.cuh"

namespace dvsgb {
namespace {

constexpr int kWarpsPerBlock = 4;  // all ray kernels launch 128 threads
// Resident blocks per SM the trace kernel is compiled for: 5 blocks of 128
// threads cap it at 96 registers (20 warps per SM), the fastest measured
// balance of latency hiding against register spills.
#ifndef DVS_TRACE_MIN_BLOCKS
#define DVS_TRACE_MIN_BLOCKS 5
#endif
constexpr int kSubrayTable = 256;  // sub-rays per pixel with a shared sub-ray table (ss <= 16)

// Element o of a radiance chunk: double, or float when the chunk feeds an
// FP32 circuit (which uses the value as a float: the same bits, half the bytes).
__device__ __forceinline__ void store_radiance(const SceneView &S, double *chunk, size_t o, double value) {
  if (S.radiance_f32) reinterpret_cast<float *>(chunk)[o] = (float)value;
  else chunk[o] = value;
}
// Several sub-rays per lane (SceneView::rays: 1, 2 or 4, when the pixel's
// sub-ray count is a multiple): the kernels with more ray state per lane are
// compiled for fewer resident blocks (more registers).
#ifndef DVS_TRACE_PAIR_MIN_BLOCKS
#define DVS_TRACE_PAIR_MIN_BLOCKS 4
#endif
#ifndef DVS_TRACE_QUAD_MIN_BLOCKS
#define DVS_TRACE_QUAD_MIN_BLOCKS 3
#endif

// One warp's share of a trace launch: warp item `warp` of the (pixel group,
// cell group) grid of one sensor -- 32/CW Morton-adjacent pixels x CW
// consecutive cells.  Called by trace_cells_kernel (one item per warp) and by
// the batch's persistent kernel (items pulled from a work counter).
template <int kMode, int kRays, int kGeo>
__device__ __forceinline__ void trace_cells_item(const SceneView &S, int n_pix, const int32_t *rank_list,
                                                 const CellPose *poses, int c0, int nc, int cw_log2,
                                                 double *radiance, float *depth_out, unsigned long long *counters,
                                                 long long warp, int *stack_code, float *stack_t,
                                                 SubraySample *subrays) {
  // n_pix pixels: all Morton ranks, or the ranks listed in rank_list
  const int lane = threadIdx.x & 31;
  const int cw = 1 << cw_log2, ppw = 32 >> cw_log2;
  const int n_groups = (nc + cw - 1) >> cw_log2;
  const long long pgroup = warp / n_groups;
  const int g = (int)(warp % n_groups);
  if (pgroup * ppw >= n_pix) return;  // warp-uniform
  const int rank = (int)(pgroup * ppw) + (lane >> cw_log2);
  const int cell = g * cw + (lane & (cw - 1));
  const bool active = rank < n_pix && cell < nc;
  const int pixel = rank < n_pix ? __ldg(S.pixel_of_rank + (rank_list ? rank_list[rank] : rank)) : 0;
  const CellPose pose = poses[c0 + (active ? cell : 0)];
  const int ss2 = S.samples * S.samples;
  // the warp's ppw pixels: their sub-rays' coordinates and FP64 cos^4 once per
  // warp (entry p * ss2 + j: sub-ray j of the pixel in lanes p * cw ...)
  const int table = ppw * ss2;
  const bool shared_subrays = kMode != kDepthOnly && table <= kSubrayTable;
  if (shared_subrays) {
    for (int q0 = 0; q0 < table; q0 += 32) {  // warp-uniform: every lane takes part in the shuffle
      const int q = q0 + lane, p = min(q / ss2, ppw - 1);
      const int pix = __shfl_sync(kFull, pixel, p << cw_log2);
      if (q < table) {
        const int j = q - p * ss2;
        const float x = subray_x(S, pix % S.width, j % S.samples), y = subray_y(S, pix / S.width, j / S.samples);
        subrays[q] = SubraySample{cos4_of(x, y), x, y};
      }
    }
    __syncwarp();
  }
  const SubraySample *mine = shared_subrays ? subrays + (lane >> cw_log2) * ss2 : nullptr;
  const PixelSample s =
      kRays > 1 ? sample_pixel_group<kMode, kRays, kGeo>(S, pixel, active, pose, stack_code, stack_t, mine)
                : sample_pixel_packet<kMode, kGeo>(S, pixel, active, pose, stack_code, stack_t, mine);
  if (active) {
    const size_t o = (size_t)cell * n_pix + rank;
    store_radiance(S, radiance, o, s.valid ? s.radiance : __longlong_as_double(0x7ff8000000000000ll));
    if (depth_out) depth_out[o] = s.depth;
  }
  const unsigned prim = warp_sum(s.primary), shad = warp_sum(s.shadow);
  if (lane == 0 && counters) {
    atomicAdd(counters + kCntPrimary, (unsigned long long)prim);
    atomicAdd(counters + kCntShadow, (unsigned long long)shad);
  }
  if (shared_subrays) __syncwarp();  // the table is rewritten by the warp's next item
}

// One pixel of a circuit launch (generate_pixels' circuit half,
// event_sensor.cu:35-50, over one cell chunk): thread r of the launch
// integrates rank rank_list[r] (or r) from radiance row r.  Called by
// circuit_kernel and by the batch's multi-sensor circuit kernel.
template <bool kF32, bool kPhilox>
__device__ __forceinline__ void circuit_rank(int r, int n, const int32_t *rank_list, const Cell *cells, int c0, int nc,
                                             const double *radiance, const PixelParams &p, const PhotoParams &photo,
                                             int max_events, const CircuitState &st, int32_t *ev_count,
                                             double *slab_t, int8_t *slab_p, int32_t *error,
                                             unsigned long long *counters) {
  const int k = rank_list ? rank_list[r] : r;
  int cnt = ev_count[k];
  if (cnt < 0) return;  // failed earlier in this batch
  const bool need_rng = !kPhilox && (photo.shot_noise || p.reset_noise_std > 0);
  curandStateXORWOW_t rng;
  if (need_rng) rng = st.rng[k];
  double *my_t = slab_t + (size_t)k * max_events;
  int8_t *my_p = slab_p + (size_t)k * max_events;
  int failed = 0;
  if (!kF32) {
    PixelRegs s{st.receptor_log[k], st.reference_log[k], st.refractory_until[k], st.threshold_pos[k],
                st.threshold_neg[k], st.reset_pending[k] != 0};
    for (int c = 0; c < nc; ++c) {
      const Cell cell = cells[c0 + c];
      const double rad = radiance[(size_t)c * n + r];
      if (!isfinite(rad)) { failed = kErrOptical; break; }
      double rate = rad * photo.electrons_per_radiance + photo.dark_electrons;
      const double t0 = cell.t0, t1 = cell.t1;
      if (photo.shot_noise) rate = poisson_electrons(rng, rate * (t1 - t0)) / (t1 - t0);
      const int emitted = advance_pixel(s, p, rate, t0, t1, my_t + cnt, my_p + cnt, max_events - cnt, rng);
      if (emitted == -1) { failed = kErrCapacity; break; }
      if (emitted == -2) { failed = kErrStalled; break; }
      cnt += emitted;
    }
    st.receptor_log[k] = s.receptor_log;
    st.reference_log[k] = s.reference_log;
    st.refractory_until[k] = s.refractory_until;
    st.reset_pending[k] = s.reset_pending ? 1 : 0;
  } else {
    // precision mode: the state is held in FP32 registers for the chunk
    PixelRegsF s{(float)st.receptor_log[k], (float)st.reference_log[k], st.refractory_until[k],
                 (float)st.threshold_pos[k], (float)st.threshold_neg[k], st.reset_pending[k] != 0, true};
    const int pixel = kPhilox ? st.pixel[k] : 0;
    const float e_rad = (float)photo.electrons_per_radiance, dark = (float)photo.dark_electrons;
    const PixelParamsF pf = pixel_params_f32(p);
    const float *chunk_f = photo.chunk_f32 ? reinterpret_cast<const float *>(radiance) : nullptr;
    for (int c = 0; c < nc; ++c) {
      const Cell cell = cells[c0 + c];
      const size_t o = (size_t)c * n + r;
      const float rad = chunk_f ? chunk_f[o] : (float)radiance[o];
      if (!isfinite(rad)) { failed = kErrOptical; break; }
      float rate = rad * e_rad + dark;
      const float dt = cell.dt;
      int emitted;
      if (kPhilox) {
        curandStatePhilox4_32_10_t ph = philox_at(photo.seed, pixel, cell.t0);
        if (photo.shot_noise) rate = poisson_electrons_philox(ph, rate * dt) / dt;
        emitted = advance_pixel_f32(s, p, pf, rate, cell.t0, dt, my_t + cnt, my_p + cnt, max_events - cnt, ph);
      } else {
        if (photo.shot_noise) rate = (float)poisson_electrons(rng, (double)(rate * dt)) / dt;
        emitted = advance_pixel_f32(s, p, pf, rate, cell.t0, dt, my_t + cnt, my_p + cnt, max_events - cnt, rng);
      }
      if (emitted == -1) { failed = kErrCapacity; break; }
      if (emitted == -2) { failed = kErrStalled; break; }
      cnt += emitted;
    }
    st.receptor_log[k] = s.receptor_log;
    st.reference_log[k] = s.reference_log;
    st.refractory_until[k] = s.refractory_until;
    st.reset_pending[k] = s.reset_pending ? 1 : 0;
  }
  if (need_rng) st.rng[k] = rng;
  if (failed) {
    atomicOr(error, failed);
    ev_count[k] = -1;
  } else {
    ev_count[k] = cnt;
  }
  if (counters && (threadIdx.x & 31) == 0) {
    const int active = min(32, n - (r & ~31));
    atomicAdd(counters + kCntCells, (unsigned long long)active * (unsigned long long)nc);
  }
}

}  // namespace
}  // namespace dvsgb
