// Device data views and kernel launchers of the GB300 DVS path.  Shared by
// kernels.cu (device code) and capi.cu (host orchestration).
#pragma once
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "dvs_internal.h"

namespace dvsgb {

struct SceneView {
  const Bvh4Node *nodes;
  const TriRecord *tris;
  const ShadeRecord *shade;
  const int32_t *pixel_of_rank;  // Morton rank -> row-major pixel index
  int32_t width, height, samples, has_albedo;
  float fx, fy, cx, cy;
  dvs_hapke hapke;
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
  int32_t pad;
};

struct PixelParams {
  double threshold_pos, threshold_neg, charge_scale, refractory_time, reference_leak, reset_noise_std;
};
struct PhotoParams {
  double electrons_per_radiance, dark_electrons, integration_step;
  int32_t shot_noise;
};

// Pixel-circuit state, structure of arrays indexed by Morton rank.
struct CircuitState {
  double *receptor_log, *reference_log, *refractory_until, *threshold_pos, *threshold_neg;
  int8_t *reset_pending;
  curandStateXORWOW_t *rng;
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

// Error word bits (host maps them to DVS_ERR_* with capacity first, as
// event_sensor.cu:300-301 tests code 1 before any other code).
enum : int32_t { kErrCapacity = 1, kErrOptical = 2, kErrStalled = 4 };

// Device counters.
enum : int { kCntPrimary = 0, kCntShadow = 1, kCntCells = 2, kCntSlots = 4 };

// ---- launchers (return cudaGetLastError()) ----------------------------------
cudaError_t launch_pose_from_state(const dvs_optical_state *state, CellPose *out, cudaStream_t s);
cudaError_t launch_cell_poses(const dvs_optical_interval *ivs, const Cell *cells, int n_cells, CellPose *out,
                              cudaStream_t s);
// Radiance (and optionally depth) of every pixel at every cell in [c0, c0+nc).
// Output index: cell * n_pix + rank.  Invalid samples store NaN radiance.
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
cudaError_t launch_radiance_to_float(int n_pix, const int32_t *pixel_of_rank, const double *radiance,
                                     const float *depth, float *image, float *depth_image, cudaStream_t s);

}  // namespace dvsgb
