// Host orchestration and C-ABI of the GB300 DVS path.
//
// dvs_scene  replaces BVHBuilder::build + DeviceScene (src/bvh/build.cpp:27-76,
//            src/cuda/device_scene.cu:15-37): one device arena holds the
//            8-wide BVH, the leaf-order triangle and shading records and the
//            Morton pixel order.
// dvs_sensor replaces EventSensor (src/cuda/event_sensor.cu:244-305): circuit
//            state in structure-of-arrays form, cuRAND XORWOW per pixel,
//            per-pixel event slabs, and the optics -> circuit chunk pipeline.
// Readout follows EventReadout (src/event_readout.cpp:6-34) on the host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "dvs_gb300.h"
#include "kernels.h"

using namespace dvsgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr, what)                                                            \
  do {                                                                                  \
    cudaError_t e__ = (expr);                                                           \
    if (e__ != cudaSuccess)                                                             \
      return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in ") + (what) + " : " +      \
                                    cudaGetErrorString(e__));                           \
  } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// parameters() and photo_parameters() (src/cuda/event_sensor.cu:151-176),
// with the compile-time switch ENABLE_PHYSIC_EFFECTS as a runtime flag.
void derive(const dvs_physic &c, bool effects, PixelParams &p, PhotoParams &photo) {
  const double q = 1.602176634e-19, k = 1.380649e-23, h = 6.62607015e-34, cl = 299792458;
  p.threshold_pos = c.threshold_pos;
  p.threshold_neg = c.threshold_neg;
  const double voltage = k * c.temperature_k / (q * c.subthreshold_kappa);
  p.charge_scale = c.receptor_capacitance_f * voltage / q;
  p.reference_leak = 0;
  p.reset_noise_std = 0;
  if (effects) {
    p.refractory_time = c.refractory_time;
    p.reference_leak = c.reset_leakage_a / (c.reset_capacitance_f * voltage);
    p.reset_noise_std = c.reset_thermal_noise ? std::sqrt(k * c.temperature_k / c.reset_capacitance_f) / voltage : 0;
  } else {
    p.refractory_time = 0;
  }
  const double pitch = c.pixel_pitch_um * 1e-6;
  const float fnum2 = 4 * c.f_number * c.f_number;  // float product, as event_sensor.cu:167
  photo.electrons_per_radiance = c.radiance_scale * 3.141592653589793 / fnum2 * c.lens_transmission * pitch * pitch *
                                 c.fill_factor * c.quantum_efficiency * (c.wavelength_nm * 1e-9) / (h * cl);
  photo.integration_step = c.circuit_step;
  if (effects) {
    photo.dark_electrons = c.dark_current_a / q;
    photo.shot_noise = c.photon_shot_noise;
  } else {
    photo.dark_electrons = 0;
    photo.shot_noise = 0;
  }
}

float material_albedo(float value, float fallback) {  // device_optics.cuh:30-33
  return std::isfinite(value) && value >= 0 && value <= 1 ? value : fallback;
}

// Morton order of the image pixels: consecutive ranks form compact 2-D tiles.
std::vector<int32_t> morton_pixel_order(int w, int h) {
  auto part = [](uint32_t v) {
    v &= 0xffff;
    v = (v | (v << 8)) & 0x00ff00ff;
    v = (v | (v << 4)) & 0x0f0f0f0f;
    v = (v | (v << 2)) & 0x33333333;
    v = (v | (v << 1)) & 0x55555555;
    return v;
  };
  std::vector<std::pair<uint32_t, int32_t>> keys((size_t)w * h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) keys[(size_t)y * w + x] = {part(x) | (part(y) << 1), y * w + x};
  std::sort(keys.begin(), keys.end());
  std::vector<int32_t> order(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) order[i] = keys[i].second;
  return order;
}

template <class T>
cudaError_t grow_device(T *&ptr, size_t &cap, size_t need) {
  if (need <= cap) return cudaSuccess;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&ptr, sizeof(T) * need);
  if (e == cudaSuccess) cap = need;
  return e;
}
template <class T>
cudaError_t grow_pinned(T *&ptr, size_t &cap, size_t need) {
  if (need <= cap) return cudaSuccess;
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMallocHost(&ptr, sizeof(T) * std::max<size_t>(need, 1));
  if (e == cudaSuccess) cap = need;
  return e;
}

}  // namespace

// Per-device set-up of dvs_cam_render_noalloc (noalloc.cu).
int dvsgb_noalloc_prepare(int device, int geometry);

// The device readout FIFO (readout.cu): its buffers in one allocation, the
// pinned status words, and the released events of the last submit or drain.
struct DeviceReadout {
  ReadoutSort sort{};
  ReadoutFifo fifo{};
  size_t max_batch = 0;
  int grid = 1;  // sort/scan blocks, sized from the previous batch
  void *arena = nullptr;
  int32_t *h_status = nullptr;  // [out_count, status]
  unsigned long long *h_counters = nullptr;  // [dropped, peak]

  cudaError_t create(double bandwidth, double latency, size_t capacity, size_t batch, cudaStream_t st) {
    max_batch = std::max<size_t>(batch, 1);
    const size_t ring = bandwidth > 0 ? next_pow2(std::min<size_t>(std::max<size_t>(capacity, 1), size_t(1) << 24))
                                      : 1;
    const int max_grid = 608;  // 4 blocks per SM of a GB300
    size_t off = 0;
    auto take = [&](size_t bytes) {
      const size_t at = off;
      off = align_up(off + bytes, 256);
      return at;
    };
    const size_t o_kt0 = take(8 * max_batch), o_kt1 = take(8 * max_batch), o_yx0 = take(4 * max_batch),
                 o_yx1 = take(4 * max_batch), o_i0 = take(4 * max_batch), o_i1 = take(4 * max_batch),
                 o_hist = take(4 * 256 * (size_t)max_grid), o_dtot = take(4 * 256), o_vary = take(8 * 3),
                 o_ring = take(sizeof(DevEvent) * ring), o_bmax = take(8 * (size_t)max_grid),
                 o_comp = take(8 * max_batch), o_del = take(8 * max_batch),
                 o_out = take(sizeof(DevEvent) * (ring + max_batch)), o_u64 = take(8 * 5), o_avail = take(8),
                 o_i32 = take(4 * 3), o_plan = take(8 * 3);
    cudaError_t e = cudaMalloc(&arena, off);
    if (e != cudaSuccess) return e;
    bytes = off;
    char *b = static_cast<char *>(arena);
    sort.kt[0] = reinterpret_cast<unsigned long long *>(b + o_kt0);
    sort.kt[1] = reinterpret_cast<unsigned long long *>(b + o_kt1);
    sort.kyx[0] = reinterpret_cast<unsigned *>(b + o_yx0);
    sort.kyx[1] = reinterpret_cast<unsigned *>(b + o_yx1);
    sort.idx[0] = reinterpret_cast<unsigned *>(b + o_i0);
    sort.idx[1] = reinterpret_cast<unsigned *>(b + o_i1);
    sort.hist = reinterpret_cast<unsigned *>(b + o_hist);
    sort.digit_total = reinterpret_cast<unsigned *>(b + o_dtot);
    sort.varying = reinterpret_cast<unsigned long long *>(b + o_vary);
    int32_t *i32 = reinterpret_cast<int32_t *>(b + o_i32);
    fifo.overflow = i32;
    fifo.status = i32 + 1;
    fifo.out_count = i32 + 2;
    unsigned long long *u64 = reinterpret_cast<unsigned long long *>(b + o_u64);
    fifo.head = u64;
    fifo.tail = u64 + 1;
    fifo.peak = u64 + 2;
    fifo.peak_batch = u64 + 3;
    fifo.dropped = u64 + 4;
    fifo.available = reinterpret_cast<double *>(b + o_avail);
    fifo.ring = reinterpret_cast<DevEvent *>(b + o_ring);
    fifo.ring_size = ring;
    fifo.capacity = capacity;
    fifo.step = bandwidth > 0 ? 1.0 / bandwidth : 0.0;
    fifo.latency = latency;
    fifo.block_max = reinterpret_cast<unsigned long long *>(b + o_bmax);
    fifo.completion = reinterpret_cast<double *>(b + o_comp);
    fifo.delivery = reinterpret_cast<double *>(b + o_del);
    fifo.plan = reinterpret_cast<long long *>(b + o_plan);
    fifo.out = reinterpret_cast<DevEvent *>(b + o_out);
    e = cudaMemsetAsync(b + o_u64, 0, o_plan + 8 * 3 - o_u64, st);  // positions, counters, availability, words
    if (e == cudaSuccess) e = cudaMallocHost(&h_status, sizeof(int32_t) * 2);
    if (e == cudaSuccess) e = cudaMallocHost(&h_counters, sizeof(unsigned long long) * 2);
    return e;
  }
  ~DeviceReadout() {
    cudaFree(arena);
    if (h_status) cudaFreeHost(h_status);
    if (h_counters) cudaFreeHost(h_counters);
  }
  static size_t next_pow2(size_t v) {
    size_t p = 1;
    while (p < v) p <<= 1;
    return p;
  }
  // Enqueues the FIFO over *count device events (none when *gate != 0) and
  // the copies of its status and counters to pinned memory.
  cudaError_t submit(const DevEvent *events, const int32_t *count, const int32_t *gate, const double *now,
                     cudaStream_t st) {
    ReadoutFifo f = fifo;
    f.gate = gate;
    cudaError_t e = launch_readout_submit(events, count, sort, f, now, grid, st);
    return e == cudaSuccess ? copy_status(st) : e;
  }
  cudaError_t drain(cudaStream_t st) {
    cudaError_t e = launch_readout_drain(fifo, grid, st);
    return e == cudaSuccess ? copy_status(st) : e;
  }
  cudaError_t copy_status(cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(h_status, fifo.out_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_status + 1, fifo.status, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_counters, fifo.dropped, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_counters + 1, fifo.peak, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    return e;
  }
  // After the stream reached the copies: the next batches' sort grid.
  void observed(size_t events) {
    grid = (int)std::min<size_t>(608, std::max<size_t>(1, (events + 4095) / 4096));
  }
  size_t bytes = 0;  // device memory held
  // kernels of one submit: keys, packing, 12 radix passes of 3, the scan's 3, commit, release, advance
  int launches() const { return readout_submit_launches(fifo.step > 0); }
};

// ---- handles --------------------------------------------------------------------
struct dvs_scene {
  int device = 0;
  dvs_camera camera{};
  int samples = 1;
  dvs_hapke hapke{};
  bool has_albedo = false;
  // geometry arena (nodes, triangle and shading records), shared by the
  // scene views created from this scene; freed with the last of them
  std::shared_ptr<void> geometry;
  size_t arena_bytes = 0;
  BvhNode *nodes = nullptr;
  BvhQNode *qnodes = nullptr;  // FP16 child bounds (nodes is then null)
  int geometry_kind = 0;       // dvs_bvh_params.precision bits
  TriRecord *tris = nullptr;
  ShadeRecord *shade = nullptr;
  int32_t *pixel_of_rank = nullptr;
  std::vector<int32_t> rank_of_pixel;  // host inverse of pixel_of_rank
  size_t n_nodes = 0, n_tris = 0, n_vertices = 0;
  int depth = 0, leaf_size = 0;
  int builder = 0;  // dvs_bvh_params.builder
  double build_seconds = 0;
  double sah_node_visits = 0, sah_triangle_tests = 0;
  float coherent_span = 1.0f;  // 0.5 % of the scene's largest extent
  // camera render buffers
  cudaStream_t stream = nullptr;
  double *cam_radiance = nullptr;
  float *cam_depth = nullptr, *cam_image = nullptr, *cam_depth_image = nullptr;
  CellPose *cam_pose = nullptr;
  dvs_optical_state *cam_state = nullptr;
  dvs_optical_state *h_state = nullptr;
  // motion-blur exposures: poses, weights and per-pose radiance, grown on demand
  size_t blur_cap = 0;
  dvs_optical_state *blur_states = nullptr, *h_blur_states = nullptr;
  float *blur_weights = nullptr, *h_blur_weights = nullptr;
  CellPose *blur_poses = nullptr;
  double *blur_radiance = nullptr;

  SceneView view() const {
    SceneView v{};  // zeroed padding: batch steps compare job tables byte for byte
    v.nodes = nodes;
    v.qnodes = qnodes;
    v.geometry = geometry_kind;
    v.tris = tris;
    v.shade = shade;
    v.pixel_of_rank = pixel_of_rank;
    v.width = camera.width;
    v.height = camera.height;
    v.samples = samples;
    v.has_albedo = has_albedo ? 1 : 0;
    v.fx = camera.fx;
    v.fy = camera.fy;
    v.cx = camera.cx;
    v.cy = camera.cy;
    v.coherent_span = coherent_span;
    v.hapke = hapke;
    v.rays = 2;
    return v;
  }
  int pixels() const { return camera.width * camera.height; }
};

struct dvs_sensor {
  dvs_scene *scene = nullptr;
  int device = 0;
  dvs_physic physic{};
  dvs_sensor_options opt{};
  PixelParams p{};
  PhotoParams photo{};
  double threshold_std = 0, threshold_min = 0;
  int max_events = 16;
  unsigned seed = 0;
  Readout *readout = nullptr;        // host FIFO (options.host_readout)
  DeviceReadout *dro = nullptr;      // device FIFO (the default)
  bool initialized = false;
  double last_time = 0;
  bool pending = false;  // an enqueued batch awaits collect
  double pending_end = 0;
  // The last upload's copies out of the pinned staging (h_ivs, h_cells) run
  // when the stream reaches them; the next batch waits for them before it
  // overwrites the staging (back-to-back enqueues stay correct).
  cudaEvent_t staged = nullptr;
  bool staged_pending = false;
  cudaStream_t stream = nullptr;
  // device state
  CircuitState st{};
  int32_t *ev_count = nullptr, *error_word = nullptr, *event_total = nullptr;
  double *slab_t = nullptr;
  int8_t *slab_p = nullptr;
  DevEvent *events = nullptr;
  unsigned long long *counters = nullptr;
  double *radiance = nullptr;
  size_t radiance_cap = 0;
  dvs_optical_interval *ivs = nullptr;
  size_t ivs_cap = 0;
  Cell *cells = nullptr;
  size_t cells_cap = 0;
  CellPose *poses = nullptr;
  size_t poses_cap = 0;
  dvs_optical_state *d_state = nullptr;
  // pinned staging
  dvs_optical_interval *h_ivs = nullptr;
  size_t h_ivs_cap = 0;
  Cell *h_cells = nullptr;
  size_t h_cells_cap = 0;
  DevEvent *h_events = nullptr;
  size_t h_events_cap = 0;
  int32_t *h_status = nullptr;  // [event_total, error]
  dvs_optical_state *h_state = nullptr;
  // results
  std::vector<HostEvent> ready;
  size_t ready_head = 0;
  dvs_sensor_stats stats{};
  // timing
  std::vector<cudaEvent_t> timers;
  size_t timers_used = 0;
  std::vector<int> timer_kind;  // 0 optics, 1 circuit, 2 events
  // adaptive optics (OpticalSampler caches, optical_sampler.hpp:305-313)
  int knot_capacity = 0;  // chosen from free memory on first use
  OpticalKnot *knots = nullptr;
  int32_t *knot_counts = nullptr, *exact_cells = nullptr, *exact_counts = nullptr, *exact_queue = nullptr;
  int32_t *exact_total = nullptr, *fallback_list = nullptr, *fallback_total = nullptr;
  double *exact_radiance = nullptr;
  unsigned long long *ref_stats = nullptr, *h_ref = nullptr;
  int32_t *probe_ranks = nullptr;
  double *probe_state = nullptr;
  int n_probes = 0;
  dvs_refinement_stats refine{};
  dvs_receptor_probe convergence{};
  // pixels this sensor owns: the whole image, or rows [row_begin, row_end)
  // (one GPU's share when several GPUs split a sensor), in Morton order
  int n_pix = 0;
  int row_begin = 0;
  const int32_t *order = nullptr;    // device: rank -> row-major pixel of the full image
  int32_t *own_order = nullptr;      // allocated when the sensor covers a row band
  std::vector<int32_t> band_rank_of_pixel;  // band-local row-major pixel -> rank
  int pixels() const { return n_pix; }
  CellPose *probe_poses = nullptr;  // the five initial adaptive probe poses
  int rays_per_lane = 2;  // traversal tuning: 1, 2 or 4 sub-rays per lane (dvs_sensor_set_tuning / autotune)
  // The view the hot path traces with: its radiance chunk is float when the
  // circuit is FP32 (photo.chunk_f32).  view64: the same with a double chunk,
  // for the initialization and the adaptive solver's knots and probes.
  SceneView view() const {
    SceneView v = view64();
    v.radiance_f32 = photo.chunk_f32;
    return v;
  }
  SceneView view64() const {
    SceneView v = scene->view();
    v.pixel_of_rank = order;
    v.rays = rays_per_lane;
    v.radiance_f32 = 0;
    return v;
  }
  size_t chunk_bytes_per_cell() const { return photo.chunk_f32 ? sizeof(float) : sizeof(double); }
};

// Accessors for the no-allocation entry point (noalloc.cu).
SceneView dvsgb_scene_view(const dvs_scene *scene) { return scene->view(); }
int dvsgb_scene_device(const dvs_scene *scene) { return scene->device; }
int dvsgb_set_error(int code, const char *message) { return fail(code, message); }

extern "C" {

const char *dvs_last_error(void) { return g_last_error.c_str(); }
const char *dvs_version(void) { return "dvs_gb300 1.0 (sm_103a)"; }

void dvs_sensor_options_default(dvs_sensor_options *out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->physic_effects = 1;
  out->aer_delay = 1;
}

int dvs_noise_poisson(int32_t generator, double lambda, uint32_t seed, size_t n, double *out) {
  if (!out || n == 0 || n > (size_t(1) << 28) || (generator != 0 && generator != 1) || !std::isfinite(lambda))
    return fail(DVS_ERR_INVALID, "invalid photon-count draw request");
  double *d = nullptr;
  cudaStream_t st = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "draw stream");
  cudaError_t e = cudaMallocAsync(&d, sizeof(double) * n, st);
  if (e == cudaSuccess) e = launch_poisson_draws(generator, lambda, seed, (int)n, 0.0, d, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (d) cudaFreeAsync(d, st);
  const cudaError_t es = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (e == cudaSuccess) e = es;
  if (e != cudaSuccess) return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in photon-count draws : ") + cudaGetErrorString(e));
  return DVS_OK;
}

int dvs_derive_parameters(const dvs_physic *physic, int32_t physic_effects, double *out9) {
  if (!physic || !out9) return fail(DVS_ERR_INVALID, "null argument");
  PixelParams p;
  PhotoParams ph;
  derive(*physic, physic_effects != 0, p, ph);
  const double v[9] = {p.threshold_pos, p.threshold_neg, p.charge_scale, p.refractory_time, p.reference_leak,
                       p.reset_noise_std, ph.electrons_per_radiance, ph.dark_electrons, ph.integration_step};
  std::memcpy(out9, v, sizeof(v));
  return DVS_OK;
}

// ---- scene ----------------------------------------------------------------------
int dvs_scene_create(const float *vertices, const float *normals, const uint32_t *indices, const float *albedos,
                     size_t n_vertices, size_t n_triangles, const dvs_camera *camera, int32_t supersample,
                     const dvs_hapke *hapke, const dvs_bvh_params *params, dvs_scene **out) {
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!vertices || !normals || !indices || !camera || !hapke || n_vertices == 0 || n_triangles == 0)
    return fail(DVS_ERR_INVALID, "invalid indexed mesh/BVH/material dimensions");
  if (camera->width <= 0 || camera->height <= 0 || camera->width > 32767 || camera->height > 32767 ||
      !(camera->fx > 0) || !(camera->fy > 0) || !std::isfinite(camera->cx) || !std::isfinite(camera->cy))
    return fail(DVS_ERR_INVALID, "invalid scene or camera range");
  if (supersample < 1 || supersample > 64 ||
      double(camera->width) * camera->height * supersample * supersample > std::numeric_limits<int>::max())
    return fail(DVS_ERR_INVALID, "too many aperture samples");
  for (size_t i = 0; i < 3 * n_vertices; ++i)
    if (!std::isfinite(vertices[i])) return fail(DVS_ERR_INVALID, "nonfinite mesh vertex");
  for (size_t i = 0; i < 3 * n_vertices; ++i)
    if (!std::isfinite(normals[i])) return fail(DVS_ERR_INVALID, "nonfinite mesh normal");
  // Default: two triangles per leaf (the fastest on terrain meshes); when the
  // tree would be too deep for the traversal stack, wider leaves.  A leaf
  // size given by the caller is used as given.
  const bool leaf_given = params && params->leaf_size > 0;
  const int precision = params ? params->precision : 0;
  if (precision < 0 || precision > 3) return fail(DVS_ERR_INVALID, "invalid BVH precision flags (0..3)");
  const int builder = params ? params->builder : 0;
  if (builder != 0 && builder != 1) return fail(DVS_ERR_INVALID, "invalid BVH builder (0 binned SAH, 1 Morton radix)");
  const bool half_bounds = precision & DVS_BVH_HALF_BOUNDS, watertight = precision & DVS_BVH_WATERTIGHT;
  BvhBuild bvh;
  std::string err;
  bool built = false;
  int leaf = leaf_given ? params->leaf_size : 2;
  for (;; leaf *= 2) {
    err.clear();
    built = build_bvh(vertices, n_vertices, indices, n_triangles, leaf, builder, bvh, err);
    if (built || leaf_given || leaf >= 8) break;
  }
  if (!built) return fail(DVS_ERR_INVALID, err);
  std::vector<BvhQNode> qnodes;
  if (half_bounds && !quantize_bvh(bvh.nodes, qnodes, err)) return fail(DVS_ERR_INVALID, err);

  // leaf-order records; a watertight scene keeps three copies of each
  // triangle's vertices, copy k in the cyclic axis order ((k+1)%3, (k+2)%3, k)
  // that the watertight test of a ray with dominant axis k reads
  const size_t copies = watertight ? 3 : 1;
  std::vector<TriRecord> tris(n_triangles * copies);
  std::vector<ShadeRecord> shade(n_triangles);
  const long long nt = (long long)n_triangles;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nt; ++i) {
    const uint32_t src = bvh.order[i];
    const uint32_t a = indices[3 * (size_t)src], b = indices[3 * (size_t)src + 1], c = indices[3 * (size_t)src + 2];
    for (size_t k = 0; k < copies; ++k) {
      TriRecord &t = tris[i * copies + k];
      std::memset(&t, 0, sizeof(t));
      const int axis[3] = {(int)(k + 1) % 3, (int)(k + 2) % 3, (int)k};
      for (int d = 0; d < 3; ++d) {
        if (watertight) {  // the vertices themselves, for the watertight test
          t.v0[d] = vertices[3 * (size_t)a + axis[d]];
          t.e1[d] = vertices[3 * (size_t)b + axis[d]];
          t.e2[d] = vertices[3 * (size_t)c + axis[d]];
        } else {
          t.v0[d] = vertices[3 * (size_t)a + d];
          t.e1[d] = vertices[3 * (size_t)b + d] - vertices[3 * (size_t)a + d];
          t.e2[d] = vertices[3 * (size_t)c + d] - vertices[3 * (size_t)a + d];
        }
      }
      t.original = src;
    }
    ShadeRecord &s = shade[i];
    std::memset(&s, 0, sizeof(s));
    for (int d = 0; d < 3; ++d) {
      s.n0[d] = normals[3 * (size_t)a + d];
      s.n1[d] = normals[3 * (size_t)b + d];
      s.n2[d] = normals[3 * (size_t)c + d];
    }
    if (albedos) {
      s.a0 = material_albedo(albedos[a], hapke->w);
      s.a1 = material_albedo(albedos[b], hapke->w);
      s.a2 = material_albedo(albedos[c], hapke->w);
    }
  }
  const std::vector<int32_t> order = morton_pixel_order(camera->width, camera->height);

  dvs_scene *s = new dvs_scene;
  s->camera = *camera;
  s->samples = supersample;
  s->hapke = *hapke;
  s->has_albedo = albedos != nullptr;
  s->n_nodes = bvh.nodes.size();
  s->n_tris = n_triangles;
  s->n_vertices = n_vertices;
  s->depth = bvh.depth;
  s->leaf_size = leaf;
  s->geometry_kind = precision;
  s->build_seconds = bvh.seconds;
  s->builder = builder;
  s->sah_node_visits = bvh.sah_node_visits;
  s->sah_triangle_tests = bvh.sah_triangle_tests;
  {
    float lo[3] = {vertices[0], vertices[1], vertices[2]}, hi[3] = {vertices[0], vertices[1], vertices[2]};
    for (size_t i = 0; i < n_vertices; ++i)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], vertices[3 * i + d]);
        hi[d] = std::max(hi[d], vertices[3 * i + d]);
      }
    s->coherent_span = 0.005f * std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1.0f});
  }
  cudaGetDevice(&s->device);
  const size_t off_nodes = 0;
  const size_t node_bytes = half_bounds ? sizeof(BvhQNode) : sizeof(BvhNode);
  const size_t off_tris = align_up(off_nodes + node_bytes * s->n_nodes, 256);
  const size_t off_shade = align_up(off_tris + sizeof(TriRecord) * tris.size(), 256);
  const size_t total = align_up(off_shade + sizeof(ShadeRecord) * n_triangles, 256);
  void *arena = nullptr;
  cudaError_t e = cudaMalloc(&arena, total);
  if (e == cudaSuccess) {
    s->geometry = std::shared_ptr<void>(arena, [](void *p) { cudaFree(p); });
    e = cudaMalloc(&s->pixel_of_rank, sizeof(int32_t) * order.size());
  }
  if (e != cudaSuccess) {
    dvs_scene_destroy(s);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in allocate scene arena : ") + cudaGetErrorString(e));
  }
  s->arena_bytes = total + sizeof(int32_t) * order.size();
  char *base = static_cast<char *>(arena);
  if (half_bounds)
    s->qnodes = reinterpret_cast<BvhQNode *>(base + off_nodes);
  else
    s->nodes = reinterpret_cast<BvhNode *>(base + off_nodes);
  s->tris = reinterpret_cast<TriRecord *>(base + off_tris);
  s->shade = reinterpret_cast<ShadeRecord *>(base + off_shade);
  s->rank_of_pixel.assign(order.size(), 0);
  for (size_t r = 0; r < order.size(); ++r) s->rank_of_pixel[order[r]] = (int32_t)r;
  if (half_bounds)
    e = cudaMemcpy(s->qnodes, qnodes.data(), sizeof(BvhQNode) * s->n_nodes, cudaMemcpyHostToDevice);
  else
    e = cudaMemcpy(s->nodes, bvh.nodes.data(), sizeof(BvhNode) * s->n_nodes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->tris, tris.data(), sizeof(TriRecord) * tris.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(s->shade, shade.data(), sizeof(ShadeRecord) * n_triangles, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(s->pixel_of_rank, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    dvs_scene_destroy(s);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in upload scene array : ") + cudaGetErrorString(e));
  }
  if (int r = dvsgb_noalloc_prepare(s->device, s->geometry_kind)) {
    dvs_scene_destroy(s);
    return r;
  }
  *out = s;
  return DVS_OK;
}

int dvs_scene_destroy(dvs_scene *s) {
  if (!s) return DVS_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaFree(s->cam_radiance);
  cudaFree(s->cam_depth);
  cudaFree(s->cam_image);
  cudaFree(s->cam_depth_image);
  cudaFree(s->cam_pose);
  cudaFree(s->cam_state);
  if (s->h_state) cudaFreeHost(s->h_state);
  cudaFree(s->blur_states);
  cudaFree(s->blur_weights);
  cudaFree(s->blur_poses);
  cudaFree(s->blur_radiance);
  if (s->h_blur_states) cudaFreeHost(s->h_blur_states);
  if (s->h_blur_weights) cudaFreeHost(s->h_blur_weights);
  if (s->stream) cudaStreamDestroy(s->stream);
  cudaFree(s->pixel_of_rank);
  s->geometry.reset();
  delete s;
  return DVS_OK;
}

int dvs_scene_view_create(const dvs_scene *base, const dvs_camera *camera, int32_t supersample,
                          const dvs_hapke *hapke, dvs_scene **out) {
  // a camera over an existing scene's geometry: one device copy of a
  // terrain's BVH serves every job that renders it
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!base || !camera || !hapke) return fail(DVS_ERR_INVALID, "invalid indexed mesh/BVH/material dimensions");
  if (camera->width <= 0 || camera->height <= 0 || camera->width > 32767 || camera->height > 32767 ||
      !(camera->fx > 0) || !(camera->fy > 0) || !std::isfinite(camera->cx) || !std::isfinite(camera->cy))
    return fail(DVS_ERR_INVALID, "invalid scene or camera range");
  if (supersample < 1 || supersample > 64 ||
      double(camera->width) * camera->height * supersample * supersample > std::numeric_limits<int>::max())
    return fail(DVS_ERR_INVALID, "too many aperture samples");
  CUDA_TRY(cudaSetDevice(base->device), "select device");
  const std::vector<int32_t> order = morton_pixel_order(camera->width, camera->height);
  dvs_scene *s = new dvs_scene;
  s->device = base->device;
  s->camera = *camera;
  s->samples = supersample;
  s->hapke = *hapke;
  s->has_albedo = base->has_albedo;
  s->geometry = base->geometry;
  s->nodes = base->nodes;
  s->qnodes = base->qnodes;
  s->geometry_kind = base->geometry_kind;
  s->tris = base->tris;
  s->shade = base->shade;
  s->n_nodes = base->n_nodes;
  s->n_tris = base->n_tris;
  s->n_vertices = base->n_vertices;
  s->depth = base->depth;
  s->leaf_size = base->leaf_size;
  s->builder = base->builder;
  s->build_seconds = base->build_seconds;
  s->sah_node_visits = base->sah_node_visits;
  s->sah_triangle_tests = base->sah_triangle_tests;
  s->coherent_span = base->coherent_span;
  s->rank_of_pixel.assign(order.size(), 0);
  for (size_t r = 0; r < order.size(); ++r) s->rank_of_pixel[order[r]] = (int32_t)r;
  cudaError_t e = cudaMalloc(&s->pixel_of_rank, sizeof(int32_t) * order.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(s->pixel_of_rank, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    dvs_scene_destroy(s);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in upload scene array : ") + cudaGetErrorString(e));
  }
  s->arena_bytes = sizeof(int32_t) * order.size();  // its own allocations; the geometry is the base's
  if (int r = dvsgb_noalloc_prepare(s->device, s->geometry_kind)) {
    dvs_scene_destroy(s);
    return r;
  }
  *out = s;
  return DVS_OK;
}

int dvs_scene_info_get(const dvs_scene *s, dvs_scene_info *out) {
  if (!s || !out) return fail(DVS_ERR_INVALID, "null argument");
  out->triangles = s->n_tris;
  out->vertices = s->n_vertices;
  out->nodes = s->n_nodes;
  out->depth = s->depth;
  out->root = 0;
  out->device_bytes = s->arena_bytes;
  out->build_seconds = s->build_seconds;
  out->leaf_size = s->leaf_size;
  out->precision = s->geometry_kind;
  out->builder = s->builder;
  out->reserved = 0;
  out->sah_node_visits = s->sah_node_visits;
  out->sah_triangle_tests = s->sah_triangle_tests;
  return DVS_OK;
}

int dvs_cam_render(dvs_scene *s, const dvs_optical_state *pose, float *radiance, float *depth) {
  if (!s || !pose || !radiance) return fail(DVS_ERR_INVALID, "invalid parallel optical request");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  const int n = s->pixels();
  if (!s->cam_radiance) {
    CUDA_TRY(cudaMalloc(&s->cam_radiance, sizeof(double) * n), "allocate optical values");
    CUDA_TRY(cudaMalloc(&s->cam_depth, sizeof(float) * n), "allocate optical depth");
    CUDA_TRY(cudaMalloc(&s->cam_image, sizeof(float) * n), "allocate image");
    CUDA_TRY(cudaMalloc(&s->cam_depth_image, sizeof(float) * n), "allocate depth image");
    CUDA_TRY(cudaMalloc(&s->cam_pose, sizeof(CellPose)), "allocate optical pose");
    CUDA_TRY(cudaMalloc(&s->cam_state, sizeof(dvs_optical_state)), "allocate optical state");
    CUDA_TRY(cudaMallocHost(&s->h_state, sizeof(dvs_optical_state)), "allocate pose staging");
  }
  *s->h_state = *pose;
  CUDA_TRY(cudaMemcpyAsync(s->cam_state, s->h_state, sizeof(dvs_optical_state), cudaMemcpyHostToDevice, s->stream),
           "upload optical poses");
  CUDA_TRY(launch_pose_from_state(s->cam_state, s->cam_pose, s->stream), "pose");
  CUDA_TRY(launch_trace_cells(s->view(), n, s->cam_pose, 0, 1, 0, s->cam_radiance, s->cam_depth, nullptr, s->stream),
           "parallel optical launch");
  CUDA_TRY(launch_radiance_to_float(n, s->pixel_of_rank, s->cam_radiance, s->cam_depth, s->cam_image,
                                    s->cam_depth_image, s->stream),
           "image layout");
  CUDA_TRY(cudaMemcpyAsync(radiance, s->cam_image, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
           "download optical values");
  if (depth)
    CUDA_TRY(cudaMemcpyAsync(depth, s->cam_depth_image, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
             "download optical depth");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "parallel optical status");
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(radiance[i])) return fail(DVS_ERR_OPTICAL, "invalid optical sample/BVH stack overflow");
  return DVS_OK;
}

int dvs_cam_render_blur(dvs_scene *s, const dvs_optical_state *poses, const float *weights, size_t n_poses,
                        float *image) {
  // main_cam_blur.cpp:64-77 with all sub-exposure poses in one multi-pose
  // launch (the pose_count form of optical_sampler.cu:154-168)
  if (!s || !poses || !weights || !image || n_poses == 0 || n_poses > (1u << 20))
    return fail(DVS_ERR_INVALID, "invalid parallel optical request");
  for (size_t j = 0; j < n_poses; ++j)
    if (!std::isfinite(weights[j])) return fail(DVS_ERR_INVALID, "invalid exposure weight");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  const int n = s->pixels();
  if (n_poses > s->blur_cap) {
    cudaStreamSynchronize(s->stream);
    cudaFree(s->blur_states);
    cudaFree(s->blur_weights);
    cudaFree(s->blur_poses);
    cudaFree(s->blur_radiance);
    if (s->h_blur_states) cudaFreeHost(s->h_blur_states);
    if (s->h_blur_weights) cudaFreeHost(s->h_blur_weights);
    s->blur_states = s->h_blur_states = nullptr;
    s->blur_weights = s->h_blur_weights = nullptr;
    s->blur_poses = nullptr;
    s->blur_radiance = nullptr;
    s->blur_cap = 0;
    CUDA_TRY(cudaMalloc(&s->blur_states, sizeof(dvs_optical_state) * n_poses), "allocate exposure poses");
    CUDA_TRY(cudaMalloc(&s->blur_weights, sizeof(float) * n_poses), "allocate exposure weights");
    CUDA_TRY(cudaMalloc(&s->blur_poses, sizeof(CellPose) * n_poses), "allocate exposure poses");
    CUDA_TRY(cudaMalloc(&s->blur_radiance, sizeof(double) * n_poses * (size_t)n), "allocate exposure radiance");
    CUDA_TRY(cudaMallocHost(&s->h_blur_states, sizeof(dvs_optical_state) * n_poses), "allocate pose staging");
    CUDA_TRY(cudaMallocHost(&s->h_blur_weights, sizeof(float) * n_poses), "allocate weight staging");
    s->blur_cap = n_poses;
  }
  if (!s->cam_image) CUDA_TRY(cudaMalloc(&s->cam_image, sizeof(float) * n), "allocate image");
  std::memcpy(s->h_blur_states, poses, sizeof(dvs_optical_state) * n_poses);
  std::memcpy(s->h_blur_weights, weights, sizeof(float) * n_poses);
  CUDA_TRY(cudaMemcpyAsync(s->blur_states, s->h_blur_states, sizeof(dvs_optical_state) * n_poses,
                           cudaMemcpyHostToDevice, s->stream),
           "upload optical poses");
  CUDA_TRY(cudaMemcpyAsync(s->blur_weights, s->h_blur_weights, sizeof(float) * n_poses, cudaMemcpyHostToDevice,
                           s->stream),
           "upload exposure weights");
  CUDA_TRY(launch_poses_from_states(s->blur_states, (int)n_poses, s->blur_poses, s->stream), "pose");
  int cw_log2 = 0;
  while (cw_log2 < 5 && (size_t(2) << cw_log2) <= n_poses) ++cw_log2;  // poses sharing a warp packet
  CUDA_TRY(launch_trace_cells(s->view(), n, s->blur_poses, 0, (int)n_poses, cw_log2, s->blur_radiance, nullptr,
                              nullptr, s->stream),
           "parallel optical launch");
  CUDA_TRY(launch_blur_accumulate(n, (int)n_poses, s->pixel_of_rank, s->blur_radiance, s->blur_weights,
                                  s->cam_image, s->stream),
           "exposure accumulation");
  CUDA_TRY(cudaMemcpyAsync(image, s->cam_image, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
           "download optical values");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "parallel optical status");
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(image[i])) return fail(DVS_ERR_OPTICAL, "invalid optical sample/BVH stack overflow");
  return DVS_OK;
}

// ---- sensor ---------------------------------------------------------------------
int dvs_sensor_destroy(dvs_sensor *s);

int dvs_sensor_create(dvs_scene *scene, const dvs_physic *physic, const dvs_sensor_options *options,
                      dvs_sensor **out) {
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!scene || !physic) return fail(DVS_ERR_INVALID, "null scene or physic configuration");
  dvs_sensor_options opt;
  if (options) opt = *options; else dvs_sensor_options_default(&opt);
  const int H = scene->camera.height, W = scene->camera.width;
  const bool band = opt.row_end > opt.row_begin;
  if (band && (opt.row_begin < 0 || opt.row_end > H))
    return fail(DVS_ERR_INVALID, "sensor row band outside the image");
  const int n = band ? (opt.row_end - opt.row_begin) * W : scene->pixels();
  if (physic->max_events_per_step < 1 || physic->max_events_per_step > 64 ||
      (long long)n * physic->max_events_per_step > std::numeric_limits<int>::max())
    return fail(DVS_ERR_INVALID, "invalid sensor capacity");
  if (!(physic->circuit_step > 0)) return fail(DVS_ERR_INVALID, "invalid optical/circuit model parameter range");
  if (opt.circuit_precision < 0 || opt.circuit_precision > 2)
    return fail(DVS_ERR_INVALID, "circuit precision must be 0 (FP64), 1 (FP32) or 2 (FP32 with Philox noise)");
  dvs_sensor *s = new dvs_sensor;
  s->scene = scene;
  s->physic = *physic;
  s->opt = opt;
  s->n_pix = n;
  s->order = scene->pixel_of_rank;
  derive(*physic, s->opt.physic_effects != 0, s->p, s->photo);
  s->photo.fp32_circuit = s->opt.circuit_precision >= 1;
  s->photo.chunk_f32 = s->photo.fp32_circuit;
  s->photo.philox = s->opt.circuit_precision == 2;
  s->photo.seed = (uint32_t)physic->random_seed;
  s->threshold_std = s->opt.physic_effects ? physic->threshold_std : 0;
  s->threshold_min = physic->threshold_min;
  s->max_events = physic->max_events_per_step;
  s->seed = (unsigned)physic->random_seed;
  s->readout = new Readout(s->opt.aer_delay ? (double)physic->readout_bandwidth : 0,
                           s->opt.aer_delay ? (double)physic->readout_latency : 0,
                           (size_t)std::max(1, physic->readout_queue_capacity));
  cudaGetDevice(&s->device);
  auto bail = [&](cudaError_t e, const char *what) {
    dvs_sensor_destroy(s);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in ") + what + " : " + cudaGetErrorString(e));
  };
  cudaError_t e;
#define ALLOC(ptr, bytes, what)                 \
  if ((e = cudaMalloc(&(ptr), (bytes))) != cudaSuccess) return bail(e, what);
  if (band) {
    // the band's pixels in the scene's Morton order; RNG subsequences and ray
    // geometry stay those of the full-image pixel
    s->row_begin = opt.row_begin;
    std::vector<int32_t> mine;
    mine.reserve(n);
    std::vector<int32_t> order_host(scene->pixels());
    for (int p = 0; p < scene->pixels(); ++p) order_host[scene->rank_of_pixel[p]] = p;
    for (int32_t p : order_host)
      if (p / W >= opt.row_begin && p / W < opt.row_end) mine.push_back(p);
    s->band_rank_of_pixel.assign(n, 0);
    for (size_t r = 0; r < mine.size(); ++r) s->band_rank_of_pixel[mine[r] - opt.row_begin * W] = (int32_t)r;
    ALLOC(s->own_order, sizeof(int32_t) * n, "sensor pixel order");
    if ((e = cudaMemcpy(s->own_order, mine.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail(e, "sensor pixel order");
    s->order = s->own_order;
  }
  ALLOC(s->st.receptor_log, sizeof(double) * n, "pixel states");
  ALLOC(s->st.reference_log, sizeof(double) * n, "pixel states");
  ALLOC(s->st.refractory_until, sizeof(double) * n, "pixel states");
  ALLOC(s->st.threshold_pos, sizeof(double) * n, "pixel states");
  ALLOC(s->st.threshold_neg, sizeof(double) * n, "pixel states");
  ALLOC(s->st.reset_pending, sizeof(int8_t) * n, "pixel states");
  ALLOC(s->st.rng, sizeof(curandStateXORWOW_t) * n, "pixel RNG");
  s->st.pixel = s->order;
  ALLOC(s->ev_count, sizeof(int32_t) * n, "event counts");
  ALLOC(s->slab_t, sizeof(double) * (size_t)n * s->max_events, "event slabs");
  ALLOC(s->slab_p, sizeof(int8_t) * (size_t)n * s->max_events, "event slabs");
  ALLOC(s->events, sizeof(DevEvent) * (size_t)n * s->max_events, "events");
  ALLOC(s->counters, sizeof(unsigned long long) * kCntSlots, "counters");
  ALLOC(s->error_word, sizeof(int32_t), "error flag");
  ALLOC(s->event_total, sizeof(int32_t), "event count");
  ALLOC(s->d_state, sizeof(dvs_optical_state), "pose");
#undef ALLOC
  if ((e = cudaMallocHost(&s->h_status, sizeof(int32_t) * 4)) != cudaSuccess) return bail(e, "status staging");
  if ((e = cudaMallocHost(&s->h_state, sizeof(dvs_optical_state))) != cudaSuccess) return bail(e, "pose staging");
  if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
  if ((e = cudaEventCreateWithFlags(&s->staged, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
  if ((e = cudaMemsetAsync(s->counters, 0, sizeof(unsigned long long) * kCntSlots, s->stream)) != cudaSuccess)
    return bail(e, "clear counters");
  if (!s->opt.host_readout) {
    s->dro = new DeviceReadout;
    if ((e = s->dro->create(s->opt.aer_delay ? (double)physic->readout_bandwidth : 0,
                            s->opt.aer_delay ? (double)physic->readout_latency : 0,
                            (size_t)std::max(1, physic->readout_queue_capacity), (size_t)n * s->max_events,
                            s->stream)) != cudaSuccess)
      return bail(e, "device readout");
  }
  *out = s;
  return DVS_OK;
}

int dvs_sensor_destroy(dvs_sensor *s) {
  if (!s) return DVS_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->staged) cudaEventDestroy(s->staged);
  cudaFree(s->st.receptor_log);
  cudaFree(s->st.reference_log);
  cudaFree(s->st.refractory_until);
  cudaFree(s->st.threshold_pos);
  cudaFree(s->st.threshold_neg);
  cudaFree(s->st.reset_pending);
  cudaFree(s->st.rng);
  cudaFree(s->ev_count);
  cudaFree(s->slab_t);
  cudaFree(s->slab_p);
  cudaFree(s->events);
  cudaFree(s->counters);
  cudaFree(s->error_word);
  cudaFree(s->event_total);
  cudaFree(s->radiance);
  cudaFree(s->ivs);
  cudaFree(s->cells);
  cudaFree(s->poses);
  cudaFree(s->probe_poses);
  cudaFree(s->d_state);
  if (s->h_ivs) cudaFreeHost(s->h_ivs);
  if (s->h_cells) cudaFreeHost(s->h_cells);
  if (s->h_events) cudaFreeHost(s->h_events);
  if (s->h_status) cudaFreeHost(s->h_status);
  if (s->h_state) cudaFreeHost(s->h_state);
  for (cudaEvent_t ev : s->timers) cudaEventDestroy(ev);
  cudaFree(s->own_order);
  cudaFree(s->knots);
  cudaFree(s->knot_counts);
  cudaFree(s->exact_cells);
  cudaFree(s->exact_counts);
  cudaFree(s->exact_queue);
  cudaFree(s->exact_total);
  cudaFree(s->exact_radiance);
  cudaFree(s->fallback_list);
  cudaFree(s->fallback_total);
  cudaFree(s->ref_stats);
  cudaFree(s->probe_ranks);
  cudaFree(s->probe_state);
  if (s->h_ref) cudaFreeHost(s->h_ref);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s->readout;
  delete s->dro;
  delete s;
  return DVS_OK;
}

void *dvs_sensor_stream(dvs_sensor *s) { return s ? (void *)s->stream : nullptr; }

static int map_error(int32_t word) {
  if (word & kErrCapacity) return fail(DVS_ERR_CAPACITY, "pixel event capacity exceeded; reduce numerical window");
  if (word & kErrOptical) return fail(DVS_ERR_OPTICAL, "invalid optical sample or BVH traversal overflow");
  if (word & kErrStalled) return fail(DVS_ERR_STALLED, "pixel circuit root solve made no progress");
  return DVS_OK;
}

// A radiance chunk of `cells` cells in the hot path's format (the buffer is
// sized in doubles; a float chunk takes half as many).
static cudaError_t ensure_radiance(dvs_sensor *s, size_t cells) {
  const size_t bytes = cells * (size_t)s->pixels() * s->chunk_bytes_per_cell();
  return grow_device(s->radiance, s->radiance_cap, (bytes + sizeof(double) - 1) / sizeof(double));
}
static cudaError_t ensure_radiance64(dvs_sensor *s, size_t cells) {
  return grow_device(s->radiance, s->radiance_cap, cells * (size_t)s->pixels());
}

int dvs_sensor_initialize(dvs_sensor *s, const dvs_optical_state *pose, double timestamp) {
  // EventSensor::initialize (event_sensor.cu:262-270)
  if (!s || !pose || !std::isfinite(timestamp) || s->initialized)
    return fail(DVS_ERR_INVALID, "invalid sensor initialization");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  const int n = s->pixels();
  CUDA_TRY(ensure_radiance64(s, 1), "initial radiance");
  CUDA_TRY(grow_device(s->poses, s->poses_cap, 1), "pose buffer");
  *s->h_state = *pose;
  CUDA_TRY(cudaMemcpyAsync(s->d_state, s->h_state, sizeof(dvs_optical_state), cudaMemcpyHostToDevice, s->stream),
           "upload pose");
  CUDA_TRY(cudaMemsetAsync(s->error_word, 0, sizeof(int32_t), s->stream), "clear initialization error");
  CUDA_TRY(launch_pose_from_state(s->d_state, s->poses, s->stream), "pose");
  CUDA_TRY(launch_trace_cells(s->view64(), n, s->poses, 0, 1, 0, s->radiance, nullptr, s->counters, s->stream),
           "initial optics");
  CUDA_TRY(launch_init_pixels(n, s->order, s->radiance, s->p, s->photo, s->threshold_std,
                              s->threshold_min, s->seed, s->st, s->error_word, s->stream),
           "initialize circuit");
  CUDA_TRY(cudaMemcpyAsync(s->h_status + 1, s->error_word, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream),
           "initialize circuit status");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "initialize circuit status");
  if (s->h_status[1]) return fail(DVS_ERR_OPTICAL, "invalid optical sample during initialization");
  s->stats.launches += 3;
  s->last_time = timestamp;
  s->initialized = true;
  return DVS_OK;
}

static void record_timer(dvs_sensor *s, int kind) {
  if (!s->opt.timing) return;
  if (s->timers_used == s->timers.size()) {
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    s->timers.push_back(ev);
    s->timer_kind.push_back(kind);
  }
  s->timer_kind[s->timers_used] = kind;
  cudaEventRecord(s->timers[s->timers_used++], s->stream);
}

// Validates the batch and builds its circuit cells in pinned staging, growing
// the device buffers they go to (upload_intervals, event_sensor.cu:274-289).
static int stage_batch(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, size_t &n_cells_out) {
  if (!s || !s->initialized || !ivs || count == 0) return fail(DVS_ERR_INVALID, "sensor not initialized or no intervals");
  if (count > (size_t)std::numeric_limits<int>::max()) return fail(DVS_ERR_INVALID, "too many intervals");
  // upload_intervals (event_sensor.cu:274-289)
  double previous = s->last_time, cells_f = 0;
  for (size_t i = 0; i < count; ++i) {
    const dvs_optical_interval &iv = ivs[i];
    if (!std::isfinite(iv.t0) || !std::isfinite(iv.t1) || iv.t0 != previous || iv.t1 <= iv.t0)
      return fail(DVS_ERR_INVALID, "sensor intervals must be positive and contiguous");
    cells_f += (iv.t1 - iv.t0) / s->photo.integration_step;
    previous = iv.t1;
  }
  if (cells_f > 1000000) return fail(DVS_ERR_INVALID, "optical horizon too long; reduce batch size");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  if (s->staged_pending) {  // the previous upload still reads the staging
    CUDA_TRY(cudaEventSynchronize(s->staged), "staging reuse");
    s->staged_pending = false;
  }
  // circuit cells, generate_pixels' loop bounds (event_sensor.cu:37-40)
  size_t n_cells = 0;
  for (size_t i = 0; i < count; ++i) n_cells += (size_t)std::ceil((ivs[i].t1 - ivs[i].t0) / s->photo.integration_step);
  CUDA_TRY(grow_pinned(s->h_cells, s->h_cells_cap, n_cells), "cell staging");
  CUDA_TRY(grow_pinned(s->h_ivs, s->h_ivs_cap, count), "interval staging");
  size_t c = 0;
  for (size_t i = 0; i < count; ++i) {
    const dvs_optical_interval &iv = ivs[i];
    const int steps = static_cast<int>(std::ceil((iv.t1 - iv.t0) / s->photo.integration_step));
    const double dt = (iv.t1 - iv.t0) / steps;
    for (int step = 0; step < steps; ++step) {
      Cell &cell = s->h_cells[c++];
      cell.t0 = iv.t0 + step * dt;
      cell.t1 = step + 1 == steps ? iv.t1 : iv.t0 + (step + 1) * dt;
      cell.interval = (int32_t)i;
      cell.dt = (float)(cell.t1 - cell.t0);
    }
  }
  std::memcpy(s->h_ivs, ivs, sizeof(dvs_optical_interval) * count);
  CUDA_TRY(grow_device(s->ivs, s->ivs_cap, count), "trajectory interval allocation");
  CUDA_TRY(grow_device(s->cells, s->cells_cap, n_cells), "cell allocation");
  CUDA_TRY(grow_device(s->poses, s->poses_cap, n_cells), "pose allocation");
  n_cells_out = n_cells;
  return DVS_OK;
}

// Uploads a staged batch and launches the per-cell pose kernel on `stream`.
// track: record when the copies have run (not inside a graph capture, where
// the batch synchronizes each step itself).
static int upload_staged(dvs_sensor *s, size_t count, size_t n_cells, cudaStream_t stream, bool track) {
  CUDA_TRY(cudaMemcpyAsync(s->ivs, s->h_ivs, sizeof(dvs_optical_interval) * count, cudaMemcpyHostToDevice, stream),
           "trajectory interval upload");
  CUDA_TRY(cudaMemcpyAsync(s->cells, s->h_cells, sizeof(Cell) * n_cells, cudaMemcpyHostToDevice, stream),
           "cell upload");
  if (track) {
    CUDA_TRY(cudaEventRecord(s->staged, stream), "staging event");
    s->staged_pending = true;
  }
  CUDA_TRY(launch_cell_poses(s->ivs, s->cells, (int)n_cells, s->poses, stream), "cell poses");
  s->stats.launches += 1;
  return DVS_OK;
}

static int upload_batch(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, size_t &n_cells_out) {
  int r = stage_batch(s, ivs, count, n_cells_out);
  return r ? r : upload_staged(s, count, n_cells_out, s->stream, true);
}

// Cells per optics launch and cells per warp packet for a batch.
static void chunk_shape(const dvs_sensor *s, size_t n_cells, size_t rows, size_t &chunk, int &cw_log2) {
  chunk = s->opt.cells_per_chunk > 0 ? (size_t)s->opt.cells_per_chunk
                                     : std::max<size_t>(1, std::min<size_t>(2048, (size_t(512) << 20) /
                                                                                   (s->chunk_bytes_per_cell() * rows)));
  chunk = std::min(chunk, n_cells);
  cw_log2 = 0;
  if (s->opt.cells_per_warp > 0) {
    while ((2 << cw_log2) <= std::min(32, s->opt.cells_per_warp)) ++cw_log2;
  } else {
    while (cw_log2 < 5 && (size_t(2) << cw_log2) <= chunk) ++cw_log2;
  }
}

static int clear_batch_outputs(dvs_sensor *s, cudaStream_t stream) {
  const int n = s->pixels();
  CUDA_TRY(cudaMemsetAsync(s->ev_count, 0, sizeof(int32_t) * n, stream), "clear events");
  CUDA_TRY(cudaMemsetAsync(s->event_total, 0, sizeof(int32_t), stream), "clear events");
  CUDA_TRY(cudaMemsetAsync(s->error_word, 0, sizeof(int32_t), stream), "clear status");
  return DVS_OK;
}

// Validates and uploads the batch, then enqueues every kernel of the hot path
// on the sensor stream without waiting (upload_intervals + generate_pixels).
static int enqueue(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count) {
  size_t n_cells = 0;
  int r = upload_batch(s, ivs, count, n_cells);
  if (r) return r;
  const int n = s->pixels();
  size_t chunk;
  int cw_log2;
  chunk_shape(s, n_cells, (size_t)n, chunk, cw_log2);
  CUDA_TRY(ensure_radiance(s, chunk), "radiance chunk allocation");
  if ((r = clear_batch_outputs(s, s->stream))) return r;
  const SceneView view = s->view();
  for (size_t c0 = 0; c0 < n_cells; c0 += chunk) {
    const int nc = (int)std::min(chunk, n_cells - c0);
    record_timer(s, 0);
    CUDA_TRY(launch_trace_cells(view, n, s->poses, (int)c0, nc, cw_log2, s->radiance, nullptr, s->counters, s->stream),
             "trace circuit cells");
    record_timer(s, 1);
    CUDA_TRY(launch_circuit(n, s->cells, (int)c0, nc, s->radiance, s->p, s->photo, s->max_events, s->st, s->ev_count,
                            s->slab_t, s->slab_p, s->error_word, s->counters, s->stream),
             "integrate circuits");
    s->stats.launches += 2;
    s->stats.optics_launches += 1;
    s->stats.circuit_launches += 1;
  }
  record_timer(s, 2);
  CUDA_TRY(launch_emit_events(n, s->order, s->scene->camera.width, s->max_events, s->ev_count,
                              s->slab_t, s->slab_p, s->events, s->event_total, s->stream),
           "compact events");
  CUDA_TRY(launch_event_depth(view, s->ivs, (int)count, s->events, s->event_total, s->error_word, s->counters,
                              s->stream),
           "event depth");
  if (s->dro) {  // the readout FIFO on the device, after the event depths
    record_timer(s, 3);
    CUDA_TRY(s->dro->submit(s->events, s->event_total, s->error_word, &s->ivs[count - 1].t1, s->stream),
             "device readout");
    s->stats.launches += s->dro->launches();
  }
  record_timer(s, 4);
  s->stats.launches += 2;
  s->last_time = ivs[count - 1].t1;
  return DVS_OK;
}

static void collect_timers(dvs_sensor *s) {
  if (!s->opt.timing) return;
  for (size_t i = 0; i + 1 < s->timers_used; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, s->timers[i], s->timers[i + 1]) != cudaSuccess) continue;
    switch (s->timer_kind[i]) {
      case 0: s->stats.optics_ms += ms; break;
      case 1: s->stats.circuit_ms += ms; break;
      case 2: s->stats.events_ms += ms; break;
      case 3: s->stats.readout_ms += ms; break;  // the device readout
      default: break;
    }
  }
  s->timers_used = 0;
}

// The device FIFO's released events (its status words already copied and
// the stream synchronized), appended to the ready list; counters updated.
static int fetch_released(dvs_sensor *s) {
  DeviceReadout &d = *s->dro;
  if (d.h_status[1]) return fail(DVS_ERR_CAPACITY, "readout queue capacity exceeds the device ring buffer");
  const int32_t released = d.h_status[0];
  if (released > 0) {
    CUDA_TRY(grow_pinned(s->h_events, s->h_events_cap, (size_t)released), "event staging");
    CUDA_TRY(cudaMemcpyAsync(s->h_events, d.fifo.out, sizeof(DevEvent) * released, cudaMemcpyDeviceToHost,
                             s->stream),
             "copy released events");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "copy released events");
  }
  for (int32_t i = 0; i < released; ++i) {
    const DevEvent &e = s->h_events[i];
    s->ready.push_back(HostEvent{e.t, e.x, e.y, e.polarity, e.depth});
  }
  s->stats.dropped = d.h_counters[0];
  s->stats.peak_queue = d.h_counters[1];
  return DVS_OK;
}

// collect_events (event_sensor.cu:296-305): status, events, readout.
static int collect(dvs_sensor *s, double end, size_t *n_ready) {
  CUDA_TRY(cudaMemcpyAsync(s->h_status, s->event_total, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream), "copy count");
  CUDA_TRY(cudaMemcpyAsync(s->h_status + 1, s->error_word, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream),
           "copy status");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "copy status");
  collect_timers(s);
  const int32_t count = s->h_status[0], word = s->h_status[1];
  if (word) return map_error(word);
  auto t0 = std::chrono::steady_clock::now();
  if (s->ready_head > 0 && s->ready_head == s->ready.size()) {
    s->ready.clear();
    s->ready_head = 0;
  }
  if (s->dro) {  // the device FIFO already ran: fetch what it released
    const size_t before = s->ready.size();
    int r = fetch_released(s);
    if (r) return r;
    s->dro->observed((size_t)count);
    s->stats.events_generated += (uint64_t)count;
    s->stats.events_delivered += s->ready.size() - before;
    if (n_ready) *n_ready = s->ready.size() - s->ready_head;
    return DVS_OK;
  }
  if (count > 0) {
    CUDA_TRY(grow_pinned(s->h_events, s->h_events_cap, (size_t)count), "event staging");
    CUDA_TRY(cudaMemcpyAsync(s->h_events, s->events, sizeof(DevEvent) * count, cudaMemcpyDeviceToHost, s->stream),
             "copy events");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "copy events");
  }
  std::vector<HostEvent> batch((size_t)count);
  for (int32_t i = 0; i < count; ++i) {
    const DevEvent &d = s->h_events[i];
    batch[i] = HostEvent{d.t, d.x, d.y, d.polarity, d.depth};
  }
  const size_t before = s->ready.size();
  s->readout->submit(batch, end, s->ready);
  s->stats.events_generated += (uint64_t)count;
  s->stats.events_delivered += s->ready.size() - before;
  s->stats.dropped = s->readout->dropped();
  s->stats.peak_queue = s->readout->peak();
  s->stats.readout_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (n_ready) *n_ready = s->ready.size() - s->ready_head;
  return DVS_OK;
}

int dvs_sensor_process(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, size_t *n_ready) {
  if (n_ready) *n_ready = 0;
  int r = enqueue(s, ivs, count);
  if (r) return r;
  s->pending = false;
  return collect(s, ivs[count - 1].t1, n_ready);
}

int dvs_sensor_enqueue(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count) {
  int r = enqueue(s, ivs, count);
  if (r) return r;
  s->pending = true;
  s->pending_end = ivs[count - 1].t1;
  return DVS_OK;
}

// ---- adaptive optics (EventSensor::process_adaptive, event_sensor.cu:306-374) ----
// Cache capacity from free memory as OpticalSampler::OpticalSampler does
// (optical_sampler.cu:141-152): 512, 256 or 128 knots per pixel.
static int ensure_adaptive(dvs_sensor *s) {
  if (s->knot_capacity) return DVS_OK;
  const size_t n = (size_t)s->pixels();
  size_t available = 0, total = 0;
  CUDA_TRY(cudaMemGetInfo(&available, &total), "query optical cache memory budget");
  int cap = 128;
  for (int candidate : {512, 256, 128}) {
    const size_t needed = n * candidate * (16 + 24 + 8 + 4);  // knot, exact cell, radiance, queue slot
    if (available > needed + (size_t(1) << 30)) {
      cap = candidate;
      break;
    }
  }
  CUDA_TRY(cudaMalloc(&s->knots, sizeof(OpticalKnot) * n * cap), "allocate pixel optical knots");
  CUDA_TRY(cudaMalloc(&s->knot_counts, sizeof(int32_t) * n), "allocate optical knot counts");
  CUDA_TRY(cudaMalloc(&s->exact_counts, sizeof(int32_t) * n), "allocate local exact cell counts");
  CUDA_TRY(cudaMalloc(&s->exact_total, sizeof(int32_t)), "allocate exact query count");
  CUDA_TRY(cudaMalloc(&s->fallback_list, sizeof(int32_t) * n), "allocate exact fallback pixel IDs");
  CUDA_TRY(cudaMalloc(&s->fallback_total, sizeof(int32_t)), "allocate exact fallback count");
  CUDA_TRY(cudaMalloc(&s->ref_stats, sizeof(unsigned long long) * kRefSlots), "allocate refinement statistics");
  CUDA_TRY(cudaMallocHost(&s->h_ref, sizeof(unsigned long long) * (kRefSlots + 4)), "refinement staging");
  // receptor-convergence probes: 1024 hashed pixels (event_sensor.cu:359-360)
  s->n_probes = (int)std::min<size_t>(1024, n);
  std::vector<int32_t> ranks(s->n_probes);
  for (int i = 0; i < s->n_probes; ++i) {
    // the sensor's i-th hashed pixel in row-major order of its own rows
    const size_t local = (size_t)((uint64_t(i) * 2654435761ULL) % n);
    const size_t pixel = (size_t)s->row_begin * s->scene->camera.width + local;
    ranks[i] = s->band_rank_of_pixel.empty() ? s->scene->rank_of_pixel[pixel]
                                             : s->band_rank_of_pixel[local];
  }
  CUDA_TRY(cudaMalloc(&s->probe_ranks, sizeof(int32_t) * s->n_probes), "allocate mean receptor probes");
  CUDA_TRY(cudaMalloc(&s->probe_state, sizeof(double) * 2 * s->n_probes), "allocate mean receptor probes");
  CUDA_TRY(cudaMemcpy(s->probe_ranks, ranks.data(), sizeof(int32_t) * s->n_probes, cudaMemcpyHostToDevice),
           "upload mean receptor probe IDs");
  s->knot_capacity = cap;
  return DVS_OK;
}

static int ensure_exact(dvs_sensor *s) {
  if (s->exact_cells) return DVS_OK;
  const size_t n = (size_t)s->pixels(), cap = (size_t)s->knot_capacity;
  CUDA_TRY(cudaMalloc(&s->exact_cells, sizeof(int32_t) * n * cap), "allocate local exact optical cells");
  CUDA_TRY(cudaMalloc(&s->exact_radiance, sizeof(double) * n * cap), "allocate local exact radiance");
  CUDA_TRY(cudaMalloc(&s->exact_queue, sizeof(int32_t) * n * cap), "allocate compact exact ray queue");
  return DVS_OK;
}

// verify_receptor (event_sensor.cu:357-374): the probe pixels' receptors
// driven by exactly traced and by interpolated light over every cell.
static int verify_receptor(dvs_sensor *s, size_t n_cells, double start, double end) {
  const SceneView view = s->view64();
  const int np = s->n_probes;
  size_t chunk;
  int cw_log2;
  chunk_shape(s, n_cells, (size_t)np, chunk, cw_log2);
  chunk = std::min(chunk, s->radiance_cap / (size_t)np);
  if (chunk == 0) chunk = 1;
  CUDA_TRY(grow_device(s->radiance, s->radiance_cap, chunk * (size_t)np), "probe radiance");
  CUDA_TRY(launch_capture_probes(np, s->probe_ranks, s->st.receptor_log, s->probe_state, s->stream),
           "capture mean receptor initial state");
  for (size_t c0 = 0; c0 < n_cells; c0 += chunk) {
    const int nc = (int)std::min(chunk, n_cells - c0);
    CUDA_TRY(launch_trace_list(view, np, s->probe_ranks, s->poses, (int)c0, nc, cw_log2, s->radiance, nullptr,
                               s->counters, s->stream),
             "mean receptor probe optics");
    CUDA_TRY(launch_advance_probes(np, s->probe_ranks, s->cells, (int)c0, nc, s->radiance, s->knots, s->knot_counts,
                                   s->knot_capacity, start, end, s->photo, s->p.charge_scale, s->probe_state,
                                   s->stream),
             "mean receptor probe integration");
    s->stats.launches += 2;
  }
  std::vector<double> states((size_t)2 * np);
  CUDA_TRY(cudaMemcpyAsync(states.data(), s->probe_state, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost, s->stream),
           "download mean receptor convergence");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "download mean receptor convergence");
  std::vector<double> errors(np);
  dvs_receptor_probe r{};
  r.pixels = np;
  r.circuit_cells = (int32_t)n_cells;
  for (int i = 0; i < np; ++i) {
    errors[i] = std::fabs(states[2 * i] - states[2 * i + 1]);
    r.mean_log_voltage_error += errors[i];
  }
  std::sort(errors.begin(), errors.end());
  r.maximum_log_voltage_error = errors.back();
  r.p99_log_voltage_error = errors[size_t(np * .99)];
  r.mean_log_voltage_error /= np;
  s->convergence = r;
  return DVS_OK;
}

int dvs_sensor_process_adaptive(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, double tolerance,
                                int32_t check_convergence, int32_t *accepted, size_t *n_ready) {
  if (accepted) *accepted = 0;
  if (n_ready) *n_ready = 0;
  if (!s || !ivs || count == 0) return fail(DVS_ERR_INVALID, "empty adaptive optical horizon");
  if (s->photo.philox)
    return fail(DVS_ERR_INVALID, "adaptive optics draws the reference's XORWOW stream; use circuit precision 0 or 1");
  const double start = ivs[0].t0, end = ivs[count - 1].t1;
  if (!std::isfinite(tolerance) || tolerance <= 0 || s->p.refractory_time <= 0 ||
      (end - start) / s->p.refractory_time + 2 > s->max_events)
    return fail(DVS_ERR_INVALID, "invalid adaptive tolerance or event capacity bound");
  size_t n_cells = 0;
  int r = upload_batch(s, ivs, count, n_cells);
  if (r) return r;
  if ((r = ensure_adaptive(s))) return r;
  const int n = s->pixels(), cap = s->knot_capacity;
  const SceneView view = s->view64();  // knots, probes and exact cells are FP64
  // all refinement completes and is checked before pixel/RNG state changes
  CUDA_TRY(cudaMemsetAsync(s->ref_stats, 0, sizeof(unsigned long long) * kRefSlots, s->stream), "clear statistics");
  CUDA_TRY(cudaMemsetAsync(s->error_word, 0, sizeof(int32_t), s->stream), "clear refinement errors");
  record_timer(s, 0);
  CUDA_TRY(ensure_radiance64(s, 5), "initial probe radiance");
  if (!s->probe_poses) CUDA_TRY(cudaMalloc(&s->probe_poses, sizeof(CellPose) * 5), "probe poses");
  CUDA_TRY(launch_refine(view, n, s->ivs, (int)count, start, end, s->photo, tolerance, s->st, s->p.charge_scale, cap,
                         s->probe_poses, s->radiance, s->knots, s->knot_counts, s->ref_stats, s->error_word,
                         s->counters, s->stream),
           "refine pixel optical launch");
  s->stats.launches += 1;
  CUDA_TRY(cudaMemcpyAsync(s->h_ref, s->ref_stats, sizeof(unsigned long long) * kRefSlots, cudaMemcpyDeviceToHost,
                           s->stream),
           "refinement statistics");
  CUDA_TRY(cudaMemcpyAsync(s->h_status + 1, s->error_word, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream),
           "refinement status");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "refinement status");
  if (s->h_status[1]) return fail(DVS_ERR_OPTICAL, "invalid ray during optical refinement");
  int32_t queries = 0;
  if (s->h_ref[kRefExactSegments]) {
    if ((r = ensure_exact(s))) return r;
    CUDA_TRY(cudaMemsetAsync(s->exact_total, 0, sizeof(int32_t), s->stream), "clear exact query queue");
    CUDA_TRY(launch_identify_exact(n, s->cells, (int)n_cells, start, end, s->knots, s->knot_counts, cap,
                                   s->exact_cells, s->exact_counts, s->exact_queue, s->exact_total, s->ref_stats,
                                   s->stream),
             "identify local exact optical cells");
    CUDA_TRY(launch_sample_exact(view, s->poses, s->exact_cells, s->exact_queue, s->exact_total, cap,
                                 s->exact_radiance, s->error_word, s->counters, s->stream),
             "trace local exact ray cells");
    s->stats.launches += 2;
    CUDA_TRY(cudaMemcpyAsync(s->h_ref, s->ref_stats, sizeof(unsigned long long) * kRefSlots, cudaMemcpyDeviceToHost,
                             s->stream),
             "local exact refinement statistics");
    CUDA_TRY(cudaMemcpyAsync(s->h_status, s->exact_total, sizeof(int32_t) * 1, cudaMemcpyDeviceToHost, s->stream),
             "local exact query count");
    CUDA_TRY(cudaMemcpyAsync(s->h_status + 1, s->error_word, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream),
             "local exact ray status");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "local exact ray status");
    if (s->h_status[1]) return fail(DVS_ERR_OPTICAL, "invalid ray in local exact optical cell");
    queries = s->h_status[0];
  }
  s->refine.traced_pixel_samples = s->h_ref[kRefTraced];
  s->refine.fallback_pixels = (int32_t)s->h_ref[kRefFallback];
  s->refine.maximum_knots = (int32_t)s->h_ref[kRefMaxKnots];
  s->refine.exact_segments = (int32_t)s->h_ref[kRefExactSegments];
  s->refine.native_cell_queries = queries;
  if (check_convergence) {
    if ((r = verify_receptor(s, n_cells, start, end))) return r;
    const double threshold = std::min(s->p.threshold_pos, s->p.threshold_neg);
    if (s->convergence.maximum_log_voltage_error > .02 * threshold ||
        s->convergence.p99_log_voltage_error > .005 * threshold) {
      collect_timers(s);
      return DVS_OK;  // rejected: no pixel, RNG or time state changed
    }
  }
  record_timer(s, 1);
  if ((r = clear_batch_outputs(s, s->stream))) return r;
  CUDA_TRY(launch_integrate_knots(n, s->cells, (int)n_cells, start, end, s->knots, s->knot_counts, cap,
                                  s->exact_cells, s->exact_radiance, queries ? s->exact_counts : nullptr, s->p,
                                  s->photo, s->max_events, s->st, s->ev_count, s->slab_t, s->slab_p, s->error_word,
                                  s->stream),
           "adaptive circuit launch");
  s->stats.launches += 1;
  const int nf = s->refine.fallback_pixels;
  if (nf > 0) {
    CUDA_TRY(cudaMemsetAsync(s->fallback_total, 0, sizeof(int32_t), s->stream), "clear fallback ID counter");
    CUDA_TRY(launch_compact_fallback(n, s->knot_counts, s->fallback_list, s->fallback_total, s->stream),
             "compact exact fallback pixels");
    size_t chunk;
    int cw_log2;
    chunk_shape(s, n_cells, (size_t)nf, chunk, cw_log2);
    CUDA_TRY(grow_device(s->radiance, s->radiance_cap, chunk * (size_t)nf), "fallback optical tile");
    for (size_t c0 = 0; c0 < n_cells; c0 += chunk) {
      const int nc = (int)std::min(chunk, n_cells - c0);
      // the fallback tile feeds the circuit: the hot path's chunk format
      CUDA_TRY(launch_trace_list(s->view(), nf, s->fallback_list, s->poses, (int)c0, nc, cw_log2, s->radiance,
                                 nullptr, s->counters, s->stream),
               "parallel exact cell optics launch");
      CUDA_TRY(launch_circuit_list(nf, s->fallback_list, s->cells, (int)c0, nc, s->radiance, s->p, s->photo,
                                   s->max_events, s->st, s->ev_count, s->slab_t, s->slab_p, s->error_word,
                                   s->counters, s->stream),
               "exact fallback circuit tile launch");
      s->stats.launches += 2;
    }
  }
  record_timer(s, 2);
  CUDA_TRY(launch_emit_events(n, s->order, s->scene->camera.width, s->max_events, s->ev_count,
                              s->slab_t, s->slab_p, s->events, s->event_total, s->stream),
           "compact events");
  if (s->dro) {
    record_timer(s, 3);
    CUDA_TRY(s->dro->submit(s->events, s->event_total, s->error_word, &s->ivs[count - 1].t1, s->stream),
             "device readout");
    s->stats.launches += s->dro->launches();
  }
  record_timer(s, 4);
  s->stats.launches += 2;
  s->last_time = end;
  if (accepted) *accepted = 1;
  return collect(s, end, n_ready);
}

int dvs_sensor_refinement_stats(const dvs_sensor *s, dvs_refinement_stats *out) {
  if (!s || !out) return fail(DVS_ERR_INVALID, "null argument");
  *out = s->refine;
  return DVS_OK;
}

int dvs_sensor_last_convergence(const dvs_sensor *s, dvs_receptor_probe *out) {
  if (!s || !out) return fail(DVS_ERR_INVALID, "null argument");
  *out = s->convergence;
  return DVS_OK;
}

int dvs_sensor_adaptive_capacity(dvs_sensor *s, int32_t *capacity) {
  if (!s || !capacity) return fail(DVS_ERR_INVALID, "null argument");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  int r = ensure_adaptive(s);
  if (r) return r;
  *capacity = s->knot_capacity;
  return DVS_OK;
}

int dvs_sensor_collect(dvs_sensor *s, size_t *n_ready) {
  if (n_ready) *n_ready = 0;
  if (!s || !s->pending) return fail(DVS_ERR_INVALID, "no enqueued batch to collect");
  s->pending = false;
  return collect(s, s->pending_end, n_ready);
}

int dvs_sensor_read(dvs_sensor *s, dvs_event *out, size_t capacity, size_t *n_out) {
  if (!s || !n_out) return fail(DVS_ERR_INVALID, "null argument");
  const size_t avail = s->ready.size() - s->ready_head;
  const size_t m = std::min(avail, capacity);
  if (m && !out) return fail(DVS_ERR_INVALID, "null output buffer");
  for (size_t i = 0; i < m; ++i) {
    const HostEvent &e = s->ready[s->ready_head + i];
    dvs_event &o = out[i];
    o.timestamp = e.t;
    o.x = e.x;
    o.y = e.y;
    o.polarity = e.p;
    o.depth = e.depth;
  }
  s->ready_head += m;
  *n_out = m;
  if (s->ready_head == s->ready.size()) {
    s->ready.clear();
    s->ready_head = 0;
  }
  return DVS_OK;
}

int dvs_sensor_process_events(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, dvs_event *out,
                              size_t capacity, size_t *n_out) {
  if (!n_out) return fail(DVS_ERR_INVALID, "null argument");
  *n_out = 0;
  size_t n_ready = 0;
  int r = dvs_sensor_process(s, ivs, count, &n_ready);
  if (r) return r;
  if (n_ready > capacity) {
    *n_out = n_ready;
    return fail(DVS_ERR_OUTPUT_SMALL, "event output buffer too small; events remain readable");
  }
  return dvs_sensor_read(s, out, capacity, n_out);
}

int dvs_sensor_drain(dvs_sensor *s, dvs_event *out, size_t capacity, size_t *n_out) {
  if (!s || !n_out) return fail(DVS_ERR_INVALID, "null argument");
  if (s->dro) {
    CUDA_TRY(cudaSetDevice(s->device), "select device");
    CUDA_TRY(s->dro->drain(s->stream), "device readout drain");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "device readout drain");
    if (s->ready_head > 0 && s->ready_head == s->ready.size()) {
      s->ready.clear();
      s->ready_head = 0;
    }
    int r = fetch_released(s);
    if (r) return r;
  } else {
    s->readout->drain(s->ready);
  }
  return dvs_sensor_read(s, out, capacity, n_out);
}

int dvs_sensor_device_bytes(const dvs_sensor *s, uint64_t *bytes) {
  if (!s || !bytes) return fail(DVS_ERR_INVALID, "null argument");
  const uint64_t n = (uint64_t)s->pixels(), ev = (uint64_t)s->max_events;
  uint64_t b = n * (5 * sizeof(double) + sizeof(int8_t) + sizeof(curandStateXORWOW_t) + sizeof(int32_t));
  b += n * ev * (sizeof(double) + sizeof(int8_t) + sizeof(DevEvent));
  b += s->radiance_cap * sizeof(double) + s->ivs_cap * sizeof(dvs_optical_interval) + s->cells_cap * sizeof(Cell) +
       s->poses_cap * sizeof(CellPose);
  if (s->own_order) b += n * sizeof(int32_t);
  if (s->knots) b += n * (uint64_t)s->knot_capacity * sizeof(OpticalKnot) + 3 * n * sizeof(int32_t);
  if (s->exact_cells) b += n * (uint64_t)s->knot_capacity * (2 * sizeof(int32_t) + sizeof(double));
  if (s->probe_state) b += (uint64_t)s->n_probes * (sizeof(int32_t) + 2 * sizeof(double));
  if (s->dro) b += s->dro->bytes;
  *bytes = b;
  return DVS_OK;
}

int dvs_sensor_stats_get(const dvs_sensor *s, dvs_sensor_stats *out) {
  if (!s || !out) return fail(DVS_ERR_INVALID, "null argument");
  unsigned long long c[kCntSlots] = {0, 0, 0, 0};
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  CUDA_TRY(cudaMemcpyAsync(c, s->counters, sizeof(c), cudaMemcpyDeviceToHost, s->stream), "copy counters");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "copy counters");
  *out = s->stats;
  out->primary_rays = c[kCntPrimary];
  out->shadow_rays = c[kCntShadow];
  out->circuit_cells = c[kCntCells];
  return DVS_OK;
}

int dvs_sensor_set_tuning(dvs_sensor *s, int32_t cells_per_warp, int32_t rays_per_lane) {
  if (!s) return fail(DVS_ERR_INVALID, "null argument");
  if (cells_per_warp < 0 || cells_per_warp > 32 || (cells_per_warp & (cells_per_warp - 1)) ||
      (rays_per_lane != 1 && rays_per_lane != 2 && rays_per_lane != 4))
    return fail(DVS_ERR_INVALID, "invalid traversal tuning");
  s->opt.cells_per_warp = cells_per_warp;
  s->rays_per_lane = rays_per_lane;
  return DVS_OK;
}

}  // extern "C"

// Second stage of the autotuner: the circuit-step chunk.  The optics ->
// circuit pipeline of every pixel over the first cells of the staged batch --
// as many as the batch's default chunk, at least 64 (or the whole batch) --
// with the chosen packet shape, for chunks of 1, 1/2, 1/4 and 1/8 of them (at
// least 4 cells), each run from the same shadow copy of the circuit state;
// the real state, RNG and time are untouched.  Keeps the default chunk unless
// another is >= 3 % faster.  (A trial of at most 64 cells could not see that a
// small sensor's whole 640-cell batch in one launch beats ten 64-cell launches:
// one launch keeps a block's consecutive packets on the same pixel.)
static int autotune_chunk(dvs_sensor *s, size_t n_cells, dvs_tuning *out) {
  const int n = s->pixels();
  size_t def_chunk;
  int cw_log2;
  chunk_shape(s, n_cells, (size_t)n, def_chunk, cw_log2);
  const int ncs = (int)std::min<size_t>(n_cells, std::max<size_t>(64, def_chunk));
  chunk_shape(s, (size_t)ncs, (size_t)n, def_chunk, cw_log2);
  std::vector<int> cands;
  for (int c = ncs; c >= 4 && cands.size() < 4; c /= 2) cands.push_back(c);
  if (std::find(cands.begin(), cands.end(), (int)def_chunk) == cands.end()) cands.push_back((int)def_chunk);
  out->cells_per_chunk = (int32_t)def_chunk;
  out->chunk_candidates = 0;
  out->chunk_cells = ncs;
  out->chunk_best_ms = out->chunk_default_ms = -1;
  if (cands.size() < 2) return DVS_OK;
  // shadow state: the five FP64 fields, the reset flags and (when drawn) the XORWOW states
  const bool rng = !s->photo.philox && (s->photo.shot_noise || s->p.reset_noise_std > 0);
  const size_t fbytes = sizeof(double) * (size_t)n, rbytes = rng ? sizeof(curandStateXORWOW_t) * (size_t)n : 0;
  char *shadow = nullptr;
  CUDA_TRY(cudaMalloc(&shadow, 5 * fbytes + (size_t)n + rbytes), "autotune shadow state");
  CircuitState st = s->st;
  double **fields[5] = {&st.receptor_log, &st.reference_log, &st.refractory_until, &st.threshold_pos,
                        &st.threshold_neg};
  double *src[5] = {s->st.receptor_log, s->st.reference_log, s->st.refractory_until, s->st.threshold_pos,
                    s->st.threshold_neg};
  for (int f = 0; f < 5; ++f) *fields[f] = reinterpret_cast<double *>(shadow + f * fbytes);
  st.reset_pending = reinterpret_cast<int8_t *>(shadow + 5 * fbytes);
  if (rng) st.rng = reinterpret_cast<curandStateXORWOW_t *>(shadow + 5 * fbytes + (size_t)n);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  if (err == cudaSuccess) err = ensure_radiance(s, (size_t)ncs);
  const SceneView view = s->view();
  float best = -1, def_ms = -1;
  int best_c = (int)def_chunk;
  for (int c : cands) {
    if (err != cudaSuccess) break;
    for (int f = 0; f < 5 && err == cudaSuccess; ++f)
      err = cudaMemcpyAsync(*fields[f], src[f], fbytes, cudaMemcpyDeviceToDevice, s->stream);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(st.reset_pending, s->st.reset_pending, (size_t)n, cudaMemcpyDeviceToDevice, s->stream);
    if (err == cudaSuccess && rng) err = cudaMemcpyAsync(st.rng, s->st.rng, rbytes, cudaMemcpyDeviceToDevice, s->stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(s->ev_count, 0, sizeof(int32_t) * n, s->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e0, s->stream);
    for (int c0 = 0; c0 < ncs && err == cudaSuccess; c0 += c) {
      const int nc = std::min(c, ncs - c0);
      err = launch_trace_cells(view, n, s->poses, c0, nc, cw_log2, s->radiance, nullptr, nullptr, s->stream);
      if (err == cudaSuccess)
        err = launch_circuit(n, s->cells, c0, nc, s->radiance, s->p, s->photo, s->max_events, st, s->ev_count,
                             s->slab_t, s->slab_p, s->error_word, nullptr, s->stream);
    }
    float ms = 0;
    if (err == cudaSuccess) err = cudaEventRecord(e1, s->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err != cudaSuccess) break;
    ++out->chunk_candidates;
    if (c == (int)def_chunk) def_ms = ms;
    if (best < 0 || ms < best) {
      best = ms;
      best_c = c;
    }
  }
  // the tuning runs leave no events or errors behind for the next batch
  if (err == cudaSuccess) err = cudaMemsetAsync(s->ev_count, 0, sizeof(int32_t) * n, s->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(s->error_word, 0, sizeof(int32_t), s->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(shadow);
  if (err != cudaSuccess) return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in chunk autotune : ") + cudaGetErrorString(err));
  if (def_ms > 0 && best > 0.97f * def_ms) {
    best = def_ms;
    best_c = (int)def_chunk;
  }
  s->opt.cells_per_chunk = best_c;
  out->cells_per_chunk = best_c;
  out->chunk_best_ms = best;
  out->chunk_default_ms = def_ms;
  return DVS_OK;
}

extern "C" {

int dvs_sensor_autotune(dvs_sensor *s, const dvs_optical_interval *ivs, size_t count, dvs_tuning *out) {
  // Times the optics of (a prefix of) the next batch for every packet shape
  // -- cells per warp 4..32, one or two sub-rays per lane -- and keeps the
  // fastest, then the circuit-step chunk (autotune_chunk).  No circuit
  // state, RNG or time changes, so the same batch is then processed as usual.
  if (!out) return fail(DVS_ERR_INVALID, "null argument");
  if (s && s->pending) return fail(DVS_ERR_INVALID, "collect the enqueued batch before autotuning");
  size_t n_cells = 0;
  int r = upload_batch(s, ivs, count, n_cells);
  if (r) return r;
  const int n = s->pixels();
  size_t chunk;
  int default_log2;
  chunk_shape(s, n_cells, (size_t)n, chunk, default_log2);
  const int nc = (int)std::min<size_t>(std::min<size_t>(chunk, n_cells), 64);
  // four patches of Morton-consecutive pixels spread over the image (at most
  // 32768 pixels in all) keep each timed launch short at any resolution
  const int n_sub = std::min(n, 32768), patch = n_sub / 4;
  std::vector<int32_t> ranks(n_sub);
  for (int i = 0; i < n_sub; ++i) {
    const int p = std::min(3, i / std::max(1, patch)), off = i - p * patch;
    ranks[i] = n_sub == n ? i : std::min(n - 1, (int)((2 * p + 1) * (long long)n / 8) + off);
  }
  int32_t *d_ranks = nullptr;
  CUDA_TRY(cudaMalloc(&d_ranks, sizeof(int32_t) * n_sub), "autotune pixels");
  cudaError_t cerr = cudaMemcpy(d_ranks, ranks.data(), sizeof(int32_t) * n_sub, cudaMemcpyHostToDevice);
  if (cerr == cudaSuccess) cerr = ensure_radiance(s, (size_t)nc);
  if (cerr != cudaSuccess) {
    cudaFree(d_ranks);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in autotune : ") + cudaGetErrorString(cerr));
  }
  const int ss2 = s->scene->samples * s->scene->samples;
  cudaEvent_t e0, e1;
  if ((cerr = cudaEventCreate(&e0)) != cudaSuccess || (cerr = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaFree(d_ranks);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in autotune timer : ") + cudaGetErrorString(cerr));
  }
  SceneView view = s->view();
  float best = -1, def_ms = -1;
  int best_log2 = default_log2, best_rays = s->rays_per_lane, tried = 0;
  cudaError_t err = cudaSuccess;
  for (int rays = 1; rays <= 4 && err == cudaSuccess; rays *= 2) {
    if (ss2 % rays) break;
    view.rays = rays;
    for (int lg = 2; lg <= 5 && err == cudaSuccess; ++lg) {
      if ((1 << lg) > nc && lg > 2) break;
      float ms = -1;
      for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {  // the first launch warms caches
        float t = 0;
        err = cudaEventRecord(e0, s->stream);
        if (err == cudaSuccess)
          err = launch_trace_list(view, n_sub, d_ranks, s->poses, 0, nc, lg, s->radiance, nullptr, nullptr,
                                  s->stream);
        if (err == cudaSuccess) err = cudaEventRecord(e1, s->stream);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && (ms < 0 || t < ms)) ms = t;
      }
      if (err != cudaSuccess) break;
      ++tried;
      if (lg == default_log2 && rays == s->rays_per_lane) def_ms = ms;
      if (best < 0 || ms < best) {
        best = ms;
        best_log2 = lg;
        best_rays = rays;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_ranks);
  if (err != cudaSuccess) return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in autotune : ") + cudaGetErrorString(err));
  if (def_ms > 0 && best > 0.97f * def_ms) {  // keep the current shape unless another is clearly faster
    best = def_ms;
    best_log2 = default_log2;
    best_rays = s->rays_per_lane;
  }
  s->opt.cells_per_warp = 1 << best_log2;
  s->rays_per_lane = best_rays;
  out->cells_per_warp = 1 << best_log2;
  out->rays_per_lane = best_rays;
  out->candidates = tried;
  out->cells_timed = nc;
  out->best_ms = best;
  out->default_ms = def_ms;
  return autotune_chunk(s, n_cells, out);
}

int dvs_sensor_stats_reset(dvs_sensor *s) {
  if (!s) return fail(DVS_ERR_INVALID, "null argument");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  CUDA_TRY(cudaMemsetAsync(s->counters, 0, sizeof(unsigned long long) * kCntSlots, s->stream), "clear counters");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "clear counters");
  const uint64_t dropped = s->stats.dropped, peak = s->stats.peak_queue;
  s->stats = dvs_sensor_stats{};
  s->stats.dropped = dropped;
  s->stats.peak_queue = peak;
  return DVS_OK;
}

int dvs_sensor_read_state(dvs_sensor *s, double *state5, int32_t *reset_pending) {
  if (!s) return fail(DVS_ERR_INVALID, "null argument");
  CUDA_TRY(cudaSetDevice(s->device), "select device");
  const int n = s->pixels();
  std::vector<double> buf((size_t)5 * n);
  std::vector<int8_t> rp(n);
  std::vector<int32_t> order(n);
  double *src[5] = {s->st.receptor_log, s->st.reference_log, s->st.refractory_until, s->st.threshold_pos,
                    s->st.threshold_neg};
  for (int f = 0; f < 5; ++f)
    CUDA_TRY(cudaMemcpyAsync(buf.data() + (size_t)f * n, src[f], sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream),
             "download state");
  CUDA_TRY(cudaMemcpyAsync(rp.data(), s->st.reset_pending, n, cudaMemcpyDeviceToHost, s->stream), "download state");
  CUDA_TRY(cudaMemcpyAsync(order.data(), s->order, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                           s->stream),
           "download order");
  CUDA_TRY(cudaStreamSynchronize(s->stream), "download state");
  const int first = s->row_begin * s->scene->camera.width;  // band sensors report their own rows
  for (int k = 0; k < n; ++k) {
    const int pix = order[k] - first;
    if (state5)
      for (int f = 0; f < 5; ++f) state5[(size_t)pix * 5 + f] = buf[(size_t)f * n + k];
    if (reset_pending) reset_pending[pix] = rp[k];
  }
  return DVS_OK;
}

}  // extern "C"

// ---- batch: many sensors over one geometry, one persistent trace per step ----------
struct dvs_batch {
  std::vector<dvs_sensor *> members;
  int device = 0;
  cudaStream_t stream = nullptr;
  // per round: the trace job table (the launch's parameter block), the circuit
  // job table (pinned staging and device copy) and the work counter
  int rounds_cap = 0;
  std::vector<TraceJobs> trace_tables;
  CircuitJob *h_circuit = nullptr, *d_circuit = nullptr;
  unsigned long long *d_next = nullptr;
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;
  // the captured step and the shape it was captured for
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> key;
  dvs_batch_stats stats{};
};

namespace {
// Everything a captured step depends on besides the job tables' contents:
// per member its activity, interval and cell counts, chunking and the device
// and pinned buffers the captured copies and launches use.
std::vector<uintptr_t> batch_key(const dvs_batch *b, const std::vector<size_t> &counts,
                                 const std::vector<size_t> &n_cells, const std::vector<size_t> &chunks,
                                 const std::vector<int> &cw, int rounds) {
  std::vector<uintptr_t> k;
  k.push_back((uintptr_t)rounds);
  for (size_t m = 0; m < b->members.size(); ++m) {
    const dvs_sensor *s = b->members[m];
    k.push_back(counts[m]);
    k.push_back(n_cells[m]);
    k.push_back(chunks[m]);
    k.push_back((uintptr_t)cw[m]);
    for (const void *ptr : {(const void *)s->h_ivs, (const void *)s->h_cells, (const void *)s->ivs,
                            (const void *)s->cells, (const void *)s->poses, (const void *)s->radiance,
                            (const void *)s->events})
      k.push_back((uintptr_t)ptr);
  }
  return k;
}
}  // namespace

extern "C" {

int dvs_batch_create(dvs_sensor *const *sensors, size_t n, dvs_batch **out) {
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!sensors || n == 0 || n > (size_t)kMaxBatchJobs)
    return fail(DVS_ERR_INVALID, "a batch holds 1 to 128 sensors");
  const void *geometry = nullptr;
  for (size_t m = 0; m < n; ++m) {
    const dvs_sensor *s = sensors[m];
    if (!s) return fail(DVS_ERR_INVALID, "null sensor in batch");
    for (size_t q = 0; q < m; ++q)
      if (sensors[q] == s) return fail(DVS_ERR_INVALID, "a sensor appears twice in the batch");
    if (m == 0) geometry = s->scene->geometry.get();
    if (s->scene->geometry.get() != geometry || s->device != sensors[0]->device)
      return fail(DVS_ERR_INVALID, "batch sensors must share one scene geometry and device");
    if (s->photo.fp32_circuit != sensors[0]->photo.fp32_circuit || s->photo.philox != sensors[0]->photo.philox)
      return fail(DVS_ERR_INVALID, "batch sensors must share one circuit precision");
  }
  CUDA_TRY(cudaSetDevice(sensors[0]->device), "select device");
  dvs_batch *b = new dvs_batch;
  b->members.assign(sensors, sensors + n);
  b->device = sensors[0]->device;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev_start);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev_end);
  if (e != cudaSuccess) {
    dvs_batch_destroy(b);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in create batch : ") + cudaGetErrorString(e));
  }
  *out = b;
  return DVS_OK;
}

int dvs_batch_destroy(dvs_batch *b) {
  if (!b) return DVS_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->h_circuit) cudaFreeHost(b->h_circuit);
  cudaFree(b->d_circuit);
  cudaFree(b->d_next);
  if (b->ev_start) cudaEventDestroy(b->ev_start);
  if (b->ev_end) cudaEventDestroy(b->ev_end);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return DVS_OK;
}

int dvs_batch_process(dvs_batch *b, const dvs_optical_interval *const *intervals, const size_t *counts,
                      size_t *n_ready) {
  if (!b || !intervals || !counts) return fail(DVS_ERR_INVALID, "null argument");
  const auto t_enter = std::chrono::steady_clock::now();
  struct HostTimer {  // host time of this call, on every return path
    dvs_batch *b;
    std::chrono::steady_clock::time_point t0;
    ~HostTimer() {
      b->stats.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  } host_timer{b, t_enter};
  const size_t n = b->members.size();
  CUDA_TRY(cudaSetDevice(b->device), "select device");
  std::vector<size_t> n_cells(n, 0), chunks(n, 0);
  std::vector<int> cw(n, 0);
  bool any = false;
  int rounds = 0;
  // a member's enqueued batch must be collected first: the step would clear
  // and overwrite the events that batch left on the device
  for (size_t m = 0; m < n; ++m)
    if (counts[m] && b->members[m]->pending)
      return fail(DVS_ERR_INVALID, "a batch member has an uncollected dvs_sensor_enqueue; collect it first");
  // stage every active member's intervals and cells; allocations happen here,
  // before any capture
  for (size_t m = 0; m < n; ++m) {
    if (n_ready) n_ready[m] = 0;
    dvs_sensor *s = b->members[m];
    if (counts[m] == 0) continue;
    if (!intervals[m]) return fail(DVS_ERR_INVALID, "null intervals for an active batch sensor");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "sensor stream");
    int r = stage_batch(s, intervals[m], counts[m], n_cells[m]);
    if (r) return r;
    chunk_shape(s, n_cells[m], (size_t)s->pixels(), chunks[m], cw[m]);
    CUDA_TRY(ensure_radiance(s, chunks[m]), "radiance chunk allocation");
    rounds = std::max(rounds, (int)((n_cells[m] + chunks[m] - 1) / chunks[m]));
    any = true;
  }
  if (!any) return DVS_OK;
  if (rounds > b->rounds_cap) {
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    b->key.clear();
    if (b->h_circuit) cudaFreeHost(b->h_circuit);
    cudaFree(b->d_circuit);
    cudaFree(b->d_next);
    b->h_circuit = nullptr; b->d_circuit = nullptr; b->d_next = nullptr;
    const size_t jobs = (size_t)rounds * kMaxBatchJobs;
    b->trace_tables.assign((size_t)rounds, TraceJobs{});
    CUDA_TRY(cudaMallocHost(&b->h_circuit, sizeof(CircuitJob) * jobs), "batch job staging");
    CUDA_TRY(cudaMalloc(&b->d_circuit, sizeof(CircuitJob) * jobs), "batch job tables");
    CUDA_TRY(cudaMalloc(&b->d_next, sizeof(unsigned long long) * rounds), "batch work counters");
    b->rounds_cap = rounds;
  }
  // the job tables of every round; rays per lane shared by the batch (2 when
  // every active member's sub-ray count is even)
  bool pairs = true;
  for (size_t m = 0; m < n; ++m)
    if (counts[m] && (b->members[m]->scene->samples * b->members[m]->scene->samples) % 2) pairs = false;
  std::vector<int> n_trace(rounds, 0), n_circuit(rounds, 0), blocks(rounds, 0);
  std::vector<long long> items(rounds, 0);
  for (int r = 0; r < rounds; ++r) {
    TraceJob *tj = b->trace_tables[r].jobs;
    std::memset(tj, 0, sizeof(TraceJob) * kMaxBatchJobs);
    CircuitJob *cj = b->h_circuit + (size_t)r * kMaxBatchJobs;
    for (size_t m = 0; m < n; ++m) {
      dvs_sensor *s = b->members[m];
      if (!counts[m]) continue;
      const size_t c0 = (size_t)r * chunks[m];
      if (c0 >= n_cells[m]) continue;
      const int nc = (int)std::min(chunks[m], n_cells[m] - c0);
      TraceJob &t = tj[n_trace[r]++];
      t.view = s->view();
      t.poses = s->poses;
      t.radiance = s->radiance;
      t.counters = s->counters;
      t.first_item = items[r];
      t.n_pix = s->pixels();
      t.c0 = (int)c0;
      t.nc = nc;
      t.cw_log2 = cw[m];
      items[r] += trace_job_items(t.n_pix, nc, cw[m]);
      CircuitJob &c = cj[n_circuit[r]++];
      c.p = s->p;
      c.photo = s->photo;
      c.st = s->st;
      c.cells = s->cells;
      c.radiance = s->radiance;
      c.ev_count = s->ev_count;
      c.slab_t = s->slab_t;
      c.slab_p = s->slab_p;
      c.error = s->error_word;
      c.counters = s->counters;
      c.n = s->pixels();
      c.c0 = (int)c0;
      c.nc = nc;
      c.max_events = s->max_events;
      c.first_block = blocks[r];
      c.pad = 0;
      blocks[r] += (c.n + 127) / 128;
    }
  }
  // capture the step once per shape; replays read the refreshed pinned tables
  std::vector<uintptr_t> key = batch_key(b, std::vector<size_t>(counts, counts + n), n_cells, chunks, cw, rounds);
  key.push_back(pairs ? 2 : 1);
  for (int r = 0; r < rounds; ++r) {
    TraceJobs &t = b->trace_tables[r];
    t.total_items = items[r];
    t.next_item = b->d_next + r;
    t.n_jobs = n_trace[r];
    t.pad = 0;
    key.push_back((uintptr_t)n_trace[r]);
    key.push_back((uintptr_t)items[r]);
    key.push_back((uintptr_t)blocks[r]);
    // the trace table is captured by value: any change in it means a new capture
    const uintptr_t *words = reinterpret_cast<const uintptr_t *>(t.jobs);
    key.insert(key.end(), words, words + sizeof(TraceJob) * n_trace[r] / sizeof(uintptr_t));
  }
  const SceneView geo = b->members[0]->view();
  const bool fp32 = b->members[0]->photo.fp32_circuit != 0, philox = b->members[0]->photo.philox != 0;
  if (!b->exec || key != b->key) {
    const auto t_capture = std::chrono::steady_clock::now();
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    cudaStream_t st = b->stream;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin batch capture");
    int rc = DVS_OK;
    // timing events as event-record nodes of the graph (a plain record inside a
    // capture only marks a dependency point)
    cudaError_t e = cudaEventRecordWithFlags(b->ev_start, st, cudaEventRecordExternal);
    for (size_t m = 0; m < n && rc == DVS_OK && e == cudaSuccess; ++m) {
      if (!counts[m]) continue;
      rc = upload_staged(b->members[m], counts[m], n_cells[m], st, false);
      if (rc == DVS_OK) rc = clear_batch_outputs(b->members[m], st);
    }
    for (int r = 0; r < rounds && rc == DVS_OK && e == cudaSuccess; ++r) {
      const size_t off = (size_t)r * kMaxBatchJobs;
      e = cudaMemcpyAsync(b->d_circuit + off, b->h_circuit + off, sizeof(CircuitJob) * n_circuit[r],
                          cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(b->d_next + r, 0, sizeof(unsigned long long), st);
      if (e == cudaSuccess) e = launch_trace_jobs(b->trace_tables[r], pairs ? 2 : 1, geo.geometry, st);
      if (e == cudaSuccess) e = launch_circuit_jobs(b->d_circuit + off, n_circuit[r], blocks[r], fp32, philox, st);
    }
    for (size_t m = 0; m < n && rc == DVS_OK && e == cudaSuccess; ++m) {
      if (!counts[m]) continue;
      dvs_sensor *s = b->members[m];
      e = launch_emit_events(s->pixels(), s->order, s->scene->camera.width, s->max_events, s->ev_count, s->slab_t,
                             s->slab_p, s->events, s->event_total, st);
      if (e == cudaSuccess)
        e = launch_event_depth(s->view(), s->ivs, (int)counts[m], s->events, s->event_total, s->error_word,
                               s->counters, st);
      if (e == cudaSuccess && s->dro)
        e = s->dro->submit(s->events, s->event_total, s->error_word, &s->ivs[counts[m] - 1].t1, st);
    }
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(b->ev_end, st, cudaEventRecordExternal);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (rc != DVS_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      b->exec = nullptr;
      b->key.clear();
      return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in capture batch step : ") + cudaGetErrorString(e));
    }
    b->key = key;
    b->stats.graph_captures += 1;
    b->stats.capture_ms +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_capture).count();
  }
  CUDA_TRY(cudaGraphLaunch(b->exec, b->stream), "launch batch step");
  CUDA_TRY(cudaStreamSynchronize(b->stream), "batch step");
  float ms = 0;
  if (cudaEventElapsedTime(&ms, b->ev_start, b->ev_end) == cudaSuccess)
    b->stats.step_ms += ms;
  else
    cudaGetLastError();  // no timing for this step; leave no error behind for the next launch check
  b->stats.steps += 1;
  b->stats.graph_launches += 1;
  b->stats.persistent_launches += (uint64_t)rounds;
  for (int r = 0; r < rounds; ++r) b->stats.trace_items += (uint64_t)items[r];
  // per member: status, events and the readout, as after a one-sensor step
  int first_error = DVS_OK;
  for (size_t m = 0; m < n; ++m) {
    if (!counts[m]) continue;
    dvs_sensor *s = b->members[m];
    s->stats.launches += 4 + (s->dro ? s->dro->launches() : 0);
    s->stats.optics_launches += 1;
    s->stats.circuit_launches += 1;
    s->last_time = intervals[m][counts[m] - 1].t1;
    s->pending = false;
    const int r = collect(s, s->last_time, n_ready ? &n_ready[m] : nullptr);
    if (r && first_error == DVS_OK) first_error = r;
  }
  return first_error;
}

int dvs_batch_stats_get(const dvs_batch *b, dvs_batch_stats *out) {
  if (!b || !out) return fail(DVS_ERR_INVALID, "null argument");
  *out = b->stats;
  return DVS_OK;
}

}  // extern "C"

// ---- standalone readout FIFO (host) -----------------------------------------------
struct dvs_readout {
  Readout fifo;
  std::vector<HostEvent> ready;
  size_t head = 0;
  dvs_readout(double b, double l, size_t c) : fifo(b, l, c) {}
};

extern "C" {

int dvs_readout_create(double bandwidth, double latency, size_t capacity, dvs_readout **out) {
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  if (!std::isfinite(bandwidth) || !std::isfinite(latency) || capacity < 1)
    return fail(DVS_ERR_INVALID, "invalid readout bandwidth, latency or capacity");
  *out = new dvs_readout(bandwidth, latency, capacity);
  return DVS_OK;
}

int dvs_readout_destroy(dvs_readout *r) {
  delete r;
  return DVS_OK;
}

static void compact_ready(dvs_readout *r) {
  if (r->head && r->head == r->ready.size()) {
    r->ready.clear();
    r->head = 0;
  }
}

int dvs_readout_submit(dvs_readout *r, const dvs_event *events, size_t n, double now, size_t *n_ready) {
  if (!r || !n_ready || (n && !events)) return fail(DVS_ERR_INVALID, "null argument");
  std::vector<HostEvent> batch(n);
  for (size_t i = 0; i < n; ++i)
    batch[i] = HostEvent{events[i].timestamp, events[i].x, events[i].y, events[i].polarity, events[i].depth};
  compact_ready(r);
  r->fifo.submit(batch, now, r->ready);
  *n_ready = r->ready.size() - r->head;
  return DVS_OK;
}

int dvs_readout_drain(dvs_readout *r, size_t *n_ready) {
  if (!r || !n_ready) return fail(DVS_ERR_INVALID, "null argument");
  compact_ready(r);
  r->fifo.drain(r->ready);
  *n_ready = r->ready.size() - r->head;
  return DVS_OK;
}

int dvs_readout_read(dvs_readout *r, dvs_event *out, size_t capacity, size_t *n_out) {
  if (!r || !n_out) return fail(DVS_ERR_INVALID, "null argument");
  const size_t m = std::min(capacity, r->ready.size() - r->head);
  if (m && !out) return fail(DVS_ERR_INVALID, "null output buffer");
  for (size_t i = 0; i < m; ++i) {
    const HostEvent &e = r->ready[r->head + i];
    out[i].timestamp = e.t;
    out[i].x = e.x;
    out[i].y = e.y;
    out[i].polarity = e.p;
    out[i].depth = e.depth;
  }
  r->head += m;
  *n_out = m;
  compact_ready(r);
  return DVS_OK;
}

int dvs_readout_counters(const dvs_readout *r, uint64_t *dropped, uint64_t *peak_queue) {
  if (!r) return fail(DVS_ERR_INVALID, "null argument");
  if (dropped) *dropped = r->fifo.dropped();
  if (peak_queue) *peak_queue = r->fifo.peak();
  return DVS_OK;
}

}  // extern "C"

// ---- standalone device readout FIFO ---------------------------------------------------
struct dvs_device_readout {
  int device = 0;
  cudaStream_t stream = nullptr;
  DeviceReadout dro;
  DevEvent *d_in = nullptr, *h_in = nullptr, *h_out = nullptr;
  int32_t *d_count = nullptr, *h_count = nullptr;
  double *d_now = nullptr, *h_now = nullptr;
  std::vector<HostEvent> ready;
  size_t head = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;  // around the kernels of the last submit
  float last_ms = 0;
};

namespace {
int device_readout_fetch(dvs_device_readout *r) {
  CUDA_TRY(cudaStreamSynchronize(r->stream), "device readout");
  if (r->dro.h_status[1]) return fail(DVS_ERR_CAPACITY, "readout queue capacity exceeds the device ring buffer");
  const int32_t released = r->dro.h_status[0];
  if (released > 0) {
    CUDA_TRY(cudaMemcpyAsync(r->h_out, r->dro.fifo.out, sizeof(DevEvent) * released, cudaMemcpyDeviceToHost,
                             r->stream),
             "copy released events");
    CUDA_TRY(cudaStreamSynchronize(r->stream), "copy released events");
  }
  if (r->head && r->head == r->ready.size()) {
    r->ready.clear();
    r->head = 0;
  }
  // host conversions of large batches run on all host threads (independent elements)
  const size_t base = r->ready.size();
  r->ready.resize(base + (size_t)std::max<int32_t>(released, 0));
  HostEvent *dst = r->ready.data() + base;
  const DevEvent *src = r->h_out;
#pragma omp parallel for schedule(static) if (released > 65536)
  for (int32_t i = 0; i < released; ++i) {
    const DevEvent &e = src[i];
    dst[i] = HostEvent{e.t, e.x, e.y, e.polarity, e.depth};
  }
  return DVS_OK;
}
}  // namespace

extern "C" {

int dvs_device_readout_create(double bandwidth, double latency, size_t capacity, size_t max_batch,
                              dvs_device_readout **out) {
  if (!out) return fail(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!std::isfinite(bandwidth) || !std::isfinite(latency) || capacity < 1 || max_batch < 1 ||
      max_batch > (size_t(1) << 28))
    return fail(DVS_ERR_INVALID, "invalid readout bandwidth, latency, capacity or batch size");
  dvs_device_readout *r = new dvs_device_readout;
  cudaGetDevice(&r->device);
  const size_t out_cap = r->dro.next_pow2(std::min<size_t>(capacity, size_t(1) << 24)) + max_batch;
  cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&r->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&r->e1);
  if (e == cudaSuccess) e = r->dro.create(bandwidth, latency, capacity, max_batch, r->stream);
  if (e == cudaSuccess) e = cudaMalloc(&r->d_in, sizeof(DevEvent) * max_batch + 64);
  if (e == cudaSuccess) e = cudaMallocHost(&r->h_in, sizeof(DevEvent) * max_batch + 64);
  if (e == cudaSuccess) e = cudaMallocHost(&r->h_out, sizeof(DevEvent) * out_cap);
  if (e == cudaSuccess) {
    r->d_count = reinterpret_cast<int32_t *>(r->d_in + max_batch);
    r->d_now = reinterpret_cast<double *>(r->d_in + max_batch) + 1;
    r->h_count = reinterpret_cast<int32_t *>(r->h_in + max_batch);
    r->h_now = reinterpret_cast<double *>(r->h_in + max_batch) + 1;
  }
  if (e != cudaSuccess) {
    dvs_device_readout_destroy(r);
    return fail(DVS_ERR_CUDA, std::string("[CUDA Error] in create device readout : ") + cudaGetErrorString(e));
  }
  *out = r;
  return DVS_OK;
}

int dvs_device_readout_destroy(dvs_device_readout *r) {
  if (!r) return DVS_OK;
  cudaSetDevice(r->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  cudaFree(r->d_in);
  if (r->h_in) cudaFreeHost(r->h_in);
  if (r->h_out) cudaFreeHost(r->h_out);
  if (r->e0) cudaEventDestroy(r->e0);
  if (r->e1) cudaEventDestroy(r->e1);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
  return DVS_OK;
}

int dvs_device_readout_submit(dvs_device_readout *r, const dvs_event *events, size_t n, double now,
                              size_t *n_ready) {
  if (!r || !n_ready || (n && !events)) return fail(DVS_ERR_INVALID, "null argument");
  if (n > r->dro.max_batch) return fail(DVS_ERR_INVALID, "more events than the readout's batch size");
  if (!std::isfinite(now)) return fail(DVS_ERR_INVALID, "invalid readout time");
  CUDA_TRY(cudaSetDevice(r->device), "select device");
#pragma omp parallel for schedule(static) if (n > 65536)
  for (long long i = 0; i < (long long)n; ++i) {
    DevEvent d{};
    d.t = events[i].timestamp;
    d.depth = events[i].depth;
    d.rank = (int32_t)i;
    d.x = events[i].x;
    d.y = events[i].y;
    d.polarity = events[i].polarity;
    r->h_in[i] = d;
  }
  *r->h_count = (int32_t)n;
  *r->h_now = now;
  if (n) CUDA_TRY(cudaMemcpyAsync(r->d_in, r->h_in, sizeof(DevEvent) * n, cudaMemcpyHostToDevice, r->stream),
                  "upload events");
  CUDA_TRY(cudaMemcpyAsync(r->d_count, r->h_count, 16, cudaMemcpyHostToDevice, r->stream), "upload count and time");
  CUDA_TRY(cudaEventRecord(r->e0, r->stream), "device readout timer");
  CUDA_TRY(r->dro.submit(r->d_in, r->d_count, nullptr, r->d_now, r->stream), "device readout");
  CUDA_TRY(cudaEventRecord(r->e1, r->stream), "device readout timer");
  int rc = device_readout_fetch(r);
  if (rc) return rc;
  CUDA_TRY(cudaEventElapsedTime(&r->last_ms, r->e0, r->e1), "device readout timer");
  r->dro.observed(n);
  *n_ready = r->ready.size() - r->head;
  return DVS_OK;
}

int dvs_device_readout_drain(dvs_device_readout *r, size_t *n_ready) {
  if (!r || !n_ready) return fail(DVS_ERR_INVALID, "null argument");
  CUDA_TRY(cudaSetDevice(r->device), "select device");
  CUDA_TRY(r->dro.drain(r->stream), "device readout drain");
  int rc = device_readout_fetch(r);
  if (rc) return rc;
  *n_ready = r->ready.size() - r->head;
  return DVS_OK;
}

int dvs_device_readout_read(dvs_device_readout *r, dvs_event *out, size_t capacity, size_t *n_out) {
  if (!r || !n_out) return fail(DVS_ERR_INVALID, "null argument");
  const size_t m = std::min(capacity, r->ready.size() - r->head);
  if (m && !out) return fail(DVS_ERR_INVALID, "null output buffer");
  const HostEvent *src = r->ready.data() + r->head;
#pragma omp parallel for schedule(static) if (m > 65536)
  for (long long i = 0; i < (long long)m; ++i) {
    const HostEvent &e = src[i];
    out[i].timestamp = e.t;
    out[i].x = e.x;
    out[i].y = e.y;
    out[i].polarity = e.p;
    out[i].depth = e.depth;
  }
  r->head += m;
  *n_out = m;
  return DVS_OK;
}

int dvs_device_readout_counters(const dvs_device_readout *r, uint64_t *dropped, uint64_t *peak_queue) {
  if (!r) return fail(DVS_ERR_INVALID, "null argument");
  if (dropped) *dropped = r->dro.h_counters[0];
  if (peak_queue) *peak_queue = r->dro.h_counters[1];
  return DVS_OK;
}

int dvs_device_readout_last_ms(const dvs_device_readout *r, double *ms) {
  if (!r || !ms) return fail(DVS_ERR_INVALID, "null argument");
  *ms = r->last_ms;
  return DVS_OK;
}

}  // extern "C"
