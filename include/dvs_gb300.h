/*
 * dvs_gb300 -- C-ABI of the GB300-native DVS hot path.
 *
 * Plain pointers and sizes only.  The structs are layout-identical to the
 * reference's device PODs so a caller can hand over the reference's own
 * vectors unchanged:
 *   dvs_optical_state    == OpticalState     (include/dvs/optical_sensor.hpp:148-152), 80 bytes
 *   dvs_optical_interval == OpticalInterval  (include/dvs/optical_sensor.hpp:153),     176 bytes
 *   dvs_event            == Event            (include/dvs/dvs_base.hpp:9-18),           17 bytes packed
 *   dvs_camera           == CameraConfig     (include/dvs/scene_types.hpp:174-177)
 *   dvs_physic           == PhysicConfig     (include/dvs/scene_types.hpp:179-194)
 *   dvs_hapke            == HapkeConfig      (include/dvs/scene_types.hpp:204-214)
 *
 * Every entry point returns a status code (DVS_OK on success); the text of the
 * last failure on the calling thread is available from dvs_last_error().  The
 * reference reports the same conditions as C++ exceptions
 * (src/cuda/event_sensor.cu:300-301, include/dvs/math_types.hpp:6-14).
 *
 * Threading: one CUDA stream per handle.  A handle is not thread-safe;
 * different handles are.  A scene may be shared by several sensors and
 * cameras (the reference shares one DeviceScene through shared_ptr) and must
 * outlive them.
 */
#ifndef DVS_GB300_H
#define DVS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define DVS_ALIGN16 alignas(16)
extern "C" {
#else
#define DVS_ALIGN16 _Alignas(16)
#endif

/* ---- status codes ------------------------------------------------------ */
#define DVS_OK 0
#define DVS_ERR_CAPACITY 1      /* "pixel event capacity exceeded; reduce numerical window" */
#define DVS_ERR_OPTICAL 2       /* "invalid optical sample or BVH traversal overflow" */
#define DVS_ERR_INVALID 3       /* invalid argument or state (std::invalid_argument) */
#define DVS_ERR_CUDA 4          /* CUDA runtime failure (std::runtime_error via CUDA_CHECK) */
#define DVS_ERR_STALLED 5       /* circuit root solve made no progress (bounded-loop guard) */
#define DVS_ERR_OUTPUT_SMALL 6  /* caller's output buffer too small; nothing was lost */

/* ---- PODs ---------------------------------------------------------------- */
typedef struct { float x, y, z; } dvs_float3;
typedef struct { DVS_ALIGN16 float x; float y, z, w; } dvs_float4; /* quaternion (x,y,z,w) */

typedef struct {
  dvs_float3 position, velocity, light, light_rate;
  dvs_float4 rotation;
  float intensity, intensity_rate;
} dvs_optical_state;

typedef struct {
  dvs_optical_state start, end;
  double t0, t1;
} dvs_optical_interval;

#pragma pack(push, 1)
typedef struct {
  double timestamp; /* seconds */
  int16_t x, y;
  int8_t polarity;  /* 1 ON, 0 OFF */
  float depth;      /* mean hit range at the event time, -1 for background */
} dvs_event;
#pragma pack(pop)

typedef struct { int32_t width, height; float fx, fy, cx, cy; } dvs_camera;

typedef struct {
  float b, c, hS, hC, thetap, w, B_S0, B_C0, phi;
} dvs_hapke;

typedef struct {
  float threshold_pos, threshold_neg, refractory_time;
  float readout_bandwidth, readout_latency;
  float threshold_std, threshold_min;
  float wavelength_nm, quantum_efficiency, pixel_pitch_um;
  float fill_factor, f_number, lens_transmission;
  float radiance_scale;
  float temperature_k, subthreshold_kappa;
  float receptor_capacitance_f;
  float reset_capacitance_f, dark_current_a;
  float reset_leakage_a, circuit_step;
  int32_t photon_shot_noise, reset_thermal_noise;
  int32_t random_seed, max_events_per_step;
  int32_t readout_queue_capacity;
} dvs_physic;

/* Runtime forms of the reference's compile-time switches
 * ENABLE_PHYSIC_EFFECTS and ENABLE_AER_DELAY (CMakeLists.txt:21-35), plus
 * the tunables of this implementation.  dvs_sensor_options_default() gives
 * the reference's defaults (both switches on). */
typedef struct {
  int32_t physic_effects;     /* shot noise, dark current, mismatch, refractory, leak, kTC */
  int32_t aer_delay;          /* finite FIFO readout */
  int32_t cells_per_chunk;    /* circuit cells traced per optics launch (0 = automatic) */
  int32_t cells_per_warp;     /* 1,2,4,8,16,32: cells sharing one warp packet (0 = automatic) */
  int32_t timing;             /* record per-kernel CUDA-event timings */
  int32_t row_begin, row_end; /* rows [row_begin, row_end) only (one GPU's share); 0,0 = all */
  int32_t circuit_precision;  /* 0: FP64 pixel circuit (reference arithmetic); 1: FP32 receptor and
                                 contrast arithmetic, FP64 times, refractory deadlines and crossing-time
                                 solves (precision mode; no counterpart in the reference); 2: as 1 with
                                 counter-based Philox noise keyed by (seed, pixel, cell index) instead of
                                 the reference's XORWOW stream (native solver only) */
  int32_t host_readout;       /* 0: the readout FIFO runs on the device (radix sort, max-plus scan of
                                 completions, pending ring buffer in device memory); 1: on the host,
                                 serially, as the reference's EventReadout */
} dvs_sensor_options;

#define DVS_BVH_HALF_BOUNDS 1
#define DVS_BVH_WATERTIGHT 2
#define DVS_BVH_BUILD_SAH 0
#define DVS_BVH_BUILD_MORTON 1
typedef struct {
  int32_t leaf_size;          /* triangles per BVH leaf, 1..8 (0: 2, wider when the tree is too deep) */
  int32_t precision;          /* geometry flags; 0 = the reference's: FP32 child bounds and its
                                 Moller-Trumbore test (device_ray.hpp:54-80).  DVS_BVH_HALF_BOUNDS:
                                 FP16 child bounds quantised outward against a per-node FP32 origin
                                 (144-byte nodes instead of 256; same hits, meshes of at most 2^27
                                 triangles).  DVS_BVH_WATERTIGHT: the watertight FP32 triangle test
                                 (Woop et al. 2013) on stored vertices.  No counterpart in the
                                 reference. */
  int32_t builder;            /* split rule of the binary tree that is collapsed to 8-wide nodes:
                                 DVS_BVH_BUILD_SAH (0, the default) = binned SAH splits with the
                                 reference's criterion (src/bvh/bining.cpp:9-103: <= 32 bins per axis,
                                 cost area x count), always split down to leaf_size;
                                 DVS_BVH_BUILD_MORTON (1) = radix splits of 63-bit Morton codes */
  int32_t reserved;
} dvs_bvh_params;

typedef struct {
  uint64_t triangles, vertices, nodes;
  int32_t depth, root;
  uint64_t device_bytes;
  double build_seconds;
  int32_t leaf_size;          /* triangles per leaf the tree was built with */
  int32_t precision;          /* dvs_bvh_params.precision flags of the tree */
  int32_t builder;            /* dvs_bvh_params.builder of the tree */
  int32_t reserved;
  double sah_node_visits;     /* surface-area model of the 8-wide tree: expected nodes visited and */
  double sah_triangle_tests;  /* triangle tests of a ray through the root box (sums of area ratios) */
} dvs_scene_info;

typedef struct {
  uint64_t primary_rays, shadow_rays;      /* traced on the device, counted there */
  uint64_t events_generated, events_delivered;
  uint64_t dropped, peak_queue;            /* readout FIFO (EventReadout::dropped/peak_queue) */
  uint64_t circuit_cells;                  /* pixel x cell integrations */
  uint64_t launches;                       /* kernels launched by this handle */
  double optics_ms, circuit_ms, events_ms;  /* device time of the kernels (options.timing) */
  double readout_ms;                        /* device time of the device readout (options.timing), or host
                                               time of the host readout */
  uint64_t optics_launches, circuit_launches;
} dvs_sensor_stats;

/* OpticalRefinementStats (include/dvs/optical_sampler.hpp:281). */
typedef struct {
  uint64_t traced_pixel_samples;
  int32_t fallback_pixels, maximum_knots, exact_segments, native_cell_queries;
} dvs_refinement_stats;

/* ReceptorProbeResult (include/dvs/event_sensor.hpp:39). */
typedef struct {
  double maximum_log_voltage_error, p99_log_voltage_error, mean_log_voltage_error;
  int32_t pixels, circuit_cells;
} dvs_receptor_probe;

typedef struct dvs_scene dvs_scene;
typedef struct dvs_sensor dvs_sensor;

/* ---- library --------------------------------------------------------------- */
const char *dvs_last_error(void);
const char *dvs_version(void);
/* Fills a default option block (reference behaviour). */
void dvs_sensor_options_default(dvs_sensor_options *out);
/* Derived per-pixel parameters, parameters()/photo_parameters()
 * (src/cuda/event_sensor.cu:151-176): out[0..5] = threshold_pos, threshold_neg,
 * charge_scale, refractory_time, reference_leak, reset_noise_std;
 * out[6..8] = electrons_per_radiance, dark_electrons, integration_step. */
int dvs_derive_parameters(const dvs_physic *physic, int32_t physic_effects, double *out9);
/* n photon counts of mean `lambda` into the host array `out`, drawn on the
 * device exactly as the circuit kernels draw them -- for distribution checks.
 * generator 0: the reference's stream, draw i from curand_init(seed, i, 0) and
 * poisson_electrons (include/dvs/photon_noise.cuh:4-9; the counts kernel of
 * tests/test_sensor.cu:17-20); generator 1: the precision mode's Philox stream
 * of pixel i for a cell starting at t = 0 (inversion below 10, Hormann's PTRS
 * up to 1e6, rounded normal above).  n <= 2^28. */
int dvs_noise_poisson(int32_t generator, double lambda, uint32_t seed, size_t n, double *out);

/* ---- scene: replaces BVHBuilder::build + DeviceScene (src/bvh/build.cpp:27-76,
 *      src/cuda/device_scene.cu:15-37) ----------------------------------------- */
/* vertices/normals: n_vertices x 3 floats; indices: n_triangles x 3 uint32;
 * albedos: n_vertices floats or NULL.  Builds the wide BVH and uploads it. */
int dvs_scene_create(const float *vertices, const float *normals, const uint32_t *indices,
                     const float *albedos, size_t n_vertices, size_t n_triangles,
                     const dvs_camera *camera, int32_t supersample, const dvs_hapke *hapke,
                     const dvs_bvh_params *params, dvs_scene **out);
int dvs_scene_destroy(dvs_scene *scene);
/* A scene with its own camera, supersampling, Hapke parameters and stream over
 * the geometry (BVH, triangle and shading records) of an existing scene: no
 * rebuild and no second device copy.  The geometry lives until the last scene
 * using it is destroyed, so base and views may be destroyed in any order.
 * Vertex albedos keep the base scene's fallback (its hapke.w).  No
 * counterpart in the reference (one DeviceScene per camera there). */
int dvs_scene_view_create(const dvs_scene *base, const dvs_camera *camera, int32_t supersample,
                          const dvs_hapke *hapke, dvs_scene **out);
int dvs_scene_info_get(const dvs_scene *scene, dvs_scene_info *out);

/* ---- camera image: replaces CamRayCaster::render_main / OpticalSampler::evaluate
 *      (src/cuda/cam_render.cu:16-28, src/cuda/optical_sampler.cu:8-23,154-168) -- */
/* radiance and depth: width*height floats each (host pointers); depth may be NULL. */
int dvs_cam_render(dvs_scene *scene, const dvs_optical_state *pose, float *radiance, float *depth);

/* Camera render that allocates no memory.  No counterpart in the reference.
 * For callers that cannot allocate device memory while rendering: a frame
 * loop under a fixed device-memory budget, a host framework that owns all
 * device memory through its own pool, or a latency-critical path where
 * cudaMalloc/cudaFree may stall or synchronize the device.
 * radiance and depth are DEVICE pointers of width*height floats (row-major;
 * depth may be NULL); the work is enqueued on `stream` (a cudaStream_t, NULL
 * for the default stream) and the call returns without waiting.  Samples that
 * could not be traced are NaN in `radiance`.
 * Intermediates live in one library-owned static device array sized for at
 * most 1280x720 pixels (about 11 MB, held on every GPU that loads the library
 * until the process exits); larger images are rejected with DVS_ERR_INVALID.
 * The per-device set-up -- looking up that array's device address and loading
 * the render's kernels, which under lazy module loading is what reserves the
 * array -- is done by dvs_scene_create / dvs_scene_view_create on the scene's
 * device, so the render itself neither allocates nor loads anything.  All
 * calls share the array: calls that overlap on the GPU race on it. */
int dvs_cam_render_noalloc(dvs_scene *scene, const dvs_optical_state *pose, float *radiance, float *depth,
                           void *stream);
/* Motion-blur exposure (apps/main_cam_blur.cpp:64-77): the image
 * sum_j weights[j] * radiance(poses[j]), accumulated in float in pose order,
 * row-major, n_poses sub-exposure poses traced in one launch (the pose_count
 * form of OpticalSampler::evaluate, src/cuda/optical_sampler.cu:154-168). */
int dvs_cam_render_blur(dvs_scene *scene, const dvs_optical_state *poses, const float *weights, size_t n_poses,
                        float *image);

/* ---- event sensor: replaces EventSensor (src/cuda/event_sensor.cu:244-305) ---- */
int dvs_sensor_create(dvs_scene *scene, const dvs_physic *physic, const dvs_sensor_options *options,
                      dvs_sensor **out);
int dvs_sensor_destroy(dvs_sensor *sensor);
/* EventSensor::initialize (event_sensor.cu:262-270). */
int dvs_sensor_initialize(dvs_sensor *sensor, const dvs_optical_state *pose, double timestamp);
/* EventSensor::process_many (event_sensor.cu:290-305): traces, integrates and
 * reads out a batch of contiguous intervals.  The ready events are kept in the
 * handle; *n_ready receives their count.  Fetch them with dvs_sensor_read. */
int dvs_sensor_process(dvs_sensor *sensor, const dvs_optical_interval *intervals, size_t n_intervals,
                       size_t *n_ready);
/* The two halves of dvs_sensor_process, for callers that overlap host work
 * with the device or time the device path alone:
 *   dvs_sensor_enqueue  validates and uploads the batch and launches every
 *                       kernel on the handle's stream without waiting; the
 *                       circuit state advances and the generated events stay
 *                       on the device;
 *   dvs_sensor_collect  waits, reports device errors, downloads the events
 *                       and runs the readout (*n_ready as in process).
 * An enqueue that is not collected before the next enqueue discards that
 * batch's events (the circuit state still advanced). */
int dvs_sensor_enqueue(dvs_sensor *sensor, const dvs_optical_interval *intervals, size_t n_intervals);
int dvs_sensor_collect(dvs_sensor *sensor, size_t *n_ready);
/* Copies up to `capacity` ready events into `out` and removes them. */
int dvs_sensor_read(dvs_sensor *sensor, dvs_event *out, size_t capacity, size_t *n_out);
/* process + read in one call; DVS_ERR_OUTPUT_SMALL leaves the events readable. */
int dvs_sensor_process_events(dvs_sensor *sensor, const dvs_optical_interval *intervals,
                              size_t n_intervals, dvs_event *out, size_t capacity, size_t *n_out);
/* EventSensor::process_adaptive (event_sensor.cu:306-355) with
 * OpticalSampler::refine / prepare_exact_cells (optical_sampler.cu:39-138,
 * 176-264): per-pixel adaptive optical knots, exact tracing of unresolved
 * cells, full native tracing of pixels whose knot cache overflows.  With
 * check_convergence the receptor-convergence gate runs first
 * (event_sensor.cu:318-326); a rejected window sets *accepted = 0 and
 * changes no pixel, RNG or time state (the caller retries, as
 * apps/main_dvs.cpp:308-312 does).  Events carry depth -1. */
int dvs_sensor_process_adaptive(dvs_sensor *sensor, const dvs_optical_interval *intervals, size_t n_intervals,
                                double log_tolerance, int32_t check_convergence, int32_t *accepted,
                                size_t *n_ready);
/* OpticalSampler::statistics / EventSensor::last_convergence / knot_capacity. */
int dvs_sensor_refinement_stats(const dvs_sensor *sensor, dvs_refinement_stats *out);
int dvs_sensor_last_convergence(const dvs_sensor *sensor, dvs_receptor_probe *out);
int dvs_sensor_adaptive_capacity(dvs_sensor *sensor, int32_t *knot_capacity);
/* EventSensor::drain / EventReadout::drain (event_readout.cpp:31-34). */
int dvs_sensor_drain(dvs_sensor *sensor, dvs_event *out, size_t capacity, size_t *n_out);
int dvs_sensor_stats_get(const dvs_sensor *sensor, dvs_sensor_stats *out);
int dvs_sensor_stats_reset(dvs_sensor *sensor);
/* ---- batch: many sensors over one scene geometry, advanced together --------------
 * No counterpart in the reference (its apps run one trajectory per process or GPU).
 * Each dvs_batch_process step traces every active member's cells in ONE persistent
 * launch -- resident blocks pull runs of work items (one warp packet of one member
 * per warp) from a device counter, so members of different sizes share the GPU
 * without a tail each --
 * and integrates every member's pixel circuits in one launch.  The step (uploads,
 * both launches, per-member event compaction and depth) is captured once into a CUDA
 * graph and replayed while the members' batch shapes stay the same; a member that
 * receives no intervals idles (the step is captured anew for the new shape).  Members
 * must share one scene geometry (dvs_scene_view_create views of one scene), device
 * and circuit_precision, and must be initialized; their events are read with
 * dvs_sensor_read as after dvs_sensor_process, and are the same as when each member
 * is processed alone.  A member may not be used outside the batch during a step, and
 * a member with an uncollected dvs_sensor_enqueue is refused (DVS_ERR_INVALID) until
 * it is collected.  The batch keeps the members' handles without owning them: every
 * member (and its scene) must outlive the batch -- destroy the batch first. */
typedef struct dvs_batch dvs_batch;
typedef struct {
  uint64_t steps, graph_launches, graph_captures, persistent_launches;
  uint64_t trace_items;       /* warp packets traced by the persistent launches */
  double step_ms;             /* device time of the steps (events at both ends of the graph) */
  double host_ms;             /* wall time inside dvs_batch_process */
  double capture_ms;          /* of which capturing and instantiating graphs */
} dvs_batch_stats;
/* 1..128 sensors. */
int dvs_batch_create(dvs_sensor *const *sensors, size_t n, dvs_batch **out);
int dvs_batch_destroy(dvs_batch *batch);
/* intervals[m], counts[m]: member m's next contiguous intervals (count 0: idle this
 * step).  n_ready (optional, n entries): events ready per member afterwards. */
int dvs_batch_process(dvs_batch *batch, const dvs_optical_interval *const *intervals, const size_t *counts,
                      size_t *n_ready);
int dvs_batch_stats_get(const dvs_batch *batch, dvs_batch_stats *out);

/* ---- standalone readout FIFO: EventReadout (include/dvs/event_sensor.hpp:24-37,
 *      src/event_readout.cpp:6-34).  Host only; used to read out event runs
 *      merged from several sensors (one per GPU) through one bus. ----------- */
typedef struct dvs_readout dvs_readout;
int dvs_readout_create(double bandwidth, double latency, size_t capacity, dvs_readout **out);
int dvs_readout_destroy(dvs_readout *readout);
/* Orders `events` by (timestamp, y, x), queues them and makes the events
 * delivered by `now` readable with dvs_readout_read (*n_ready = how many). */
int dvs_readout_submit(dvs_readout *readout, const dvs_event *events, size_t n_events, double now,
                       size_t *n_ready);
int dvs_readout_drain(dvs_readout *readout, size_t *n_ready);
int dvs_readout_read(dvs_readout *readout, dvs_event *out, size_t capacity, size_t *n_out);
int dvs_readout_counters(const dvs_readout *readout, uint64_t *dropped, uint64_t *peak_queue);

/* ---- the same FIFO on the device: EventReadout::submit/drain
 *      (src/event_readout.cpp:6-34) as a stable radix sort by (t, y, x), a
 *      max-plus scan of the completions, per-arrival occupancy by binary search
 *      (a bounded serial pass on the device when the queue fills) and a pending
 *      ring buffer in device memory.  Sensors use it unless
 *      dvs_sensor_options.host_readout is set; this handle reads out a host
 *      array of up to max_batch events per submit.  Order, drops and peak are
 *      the serial FIFO's; delivery times equal them up to FP64 rounding. ---- */
typedef struct dvs_device_readout dvs_device_readout;
int dvs_device_readout_create(double bandwidth, double latency, size_t capacity, size_t max_batch,
                              dvs_device_readout **out);
int dvs_device_readout_destroy(dvs_device_readout *readout);
int dvs_device_readout_submit(dvs_device_readout *readout, const dvs_event *events, size_t n_events, double now,
                              size_t *n_ready);
int dvs_device_readout_drain(dvs_device_readout *readout, size_t *n_ready);
int dvs_device_readout_read(dvs_device_readout *readout, dvs_event *out, size_t capacity, size_t *n_out);
int dvs_device_readout_counters(const dvs_device_readout *readout, uint64_t *dropped, uint64_t *peak_queue);
/* Device time of the last submit's kernels (CUDA events on the handle's stream). */
int dvs_device_readout_last_ms(const dvs_device_readout *readout, double *ms);

/* Traversal packet shape: cells_per_warp 1..32 (power of two; 0 = automatic)
 * and rays_per_lane 1, 2 (the default) or 4 neighbouring sub-rays per lane,
 * used when the pixel's sub-ray count is a multiple of it. */
int dvs_sensor_set_tuning(dvs_sensor *sensor, int32_t cells_per_warp, int32_t rays_per_lane);
typedef struct {
  int32_t cells_per_warp, rays_per_lane;  /* the shape chosen and now set */
  int32_t candidates, cells_timed;        /* shapes timed, circuit cells in the timed launch */
  double best_ms, default_ms;             /* trace time of the chosen shape and of the previous one */
  int32_t cells_per_chunk;                /* circuit-step chunk chosen and now set (cells per optics launch) */
  int32_t chunk_candidates, chunk_cells;  /* chunk sizes timed, cells of the timed pipeline */
  double chunk_best_ms, chunk_default_ms; /* optics + circuit time of the chosen and of the previous chunk */
} dvs_tuning;
/* Autotuner, two stages, both on a prefix of the next batch (the intervals
 * dvs_sensor_process/enqueue will be given next):
 *  1. packet shape: the trace of up to 64 circuit cells over a patch of up
 *     to 32768 pixels from the middle of the image, for each shape (cells per
 *     warp 4..32 x 1, 2 or 4 sub-rays per lane);
 *  2. circuit-step chunking: the whole optics -> circuit pipeline of every
 *     pixel with the chosen shape over as many cells as the batch's default
 *     chunk (at least 64, at most the batch), for chunks of 1, 1/2, 1/4 and
 *     1/8 of them (at least 4 cells), on a shadow copy of the circuit state --
 *     smaller chunks keep the radiance of a launch in L2 for the circuit,
 *     larger ones launch less and keep a block's packets on one pixel.
 * Each stage keeps the current setting unless another is >= 3 % faster.  No
 * circuit state, RNG or time changes; not allowed while an enqueued batch
 * awaits collect. */
int dvs_sensor_autotune(dvs_sensor *sensor, const dvs_optical_interval *intervals, size_t n_intervals,
                        dvs_tuning *out);
/* Device memory the sensor holds now (state, RNG, event slabs, radiance
 * chunk, batch buffers, adaptive caches), for admission by a memory budget. */
int dvs_sensor_device_bytes(const dvs_sensor *sensor, uint64_t *bytes);
/* The CUDA stream (cudaStream_t) the handle launches on, for external timing. */
void *dvs_sensor_stream(dvs_sensor *sensor);
/* Per-pixel circuit state in row-major order of the sensor's rows: 5 doubles per pixel
 * (receptor_log, reference_log, refractory_until, threshold_pos, threshold_neg)
 * and one int32 reset flag.  Either pointer may be NULL. */
int dvs_sensor_read_state(dvs_sensor *sensor, double *state5, int32_t *reset_pending);

/* ---- host inputs of bin/dvs and bin/cam ------------------------------------------
 * The YAML config (src/scene_types.cpp:170-345), the frames.bin trajectory of a
 * scene bundle (src/scene_data.cpp:163-193) and the continuous camera/light
 * trajectory (src/trajectory.cpp), restated in C++ without Eigen.  Host only:
 * these calls need no GPU. */
typedef struct {
  int32_t frame_count;
  float fps, imu_fps, cam_fps, time_resolution, blur_resolution;
  int32_t supersample_factor;
  float translation[3], rotation[3]; /* camera mount in the trajectory frame; Euler X, Y, Z (radians) */
} dvs_scene_config;

typedef struct {
  int32_t frame_index;
  double timestamp_seconds;   /* NaN: the frame's time is frame_index / fps */
  float camera_origin[3];
  float camera_world[9];      /* row-major camera-to-world rotation */
  float light_dir[3];
  float light_intensity;
} dvs_frame;

typedef struct dvs_trajectory dvs_trajectory;

/* Parses a config file; DVS_ERR_INVALID with the reference's message when it
 * is missing, malformed or out of range.  Any output pointer may be NULL. */
int dvs_config_load(const char *path, dvs_camera *camera, dvs_physic *physic, dvs_hapke *hapke,
                    dvs_scene_config *scene);
/* Reads <bundle_dir>/frames.bin.  *n_frames = frames in the file; copies
 * min(capacity, n) of them; frames == NULL queries the count.
 * DVS_ERR_OUTPUT_SMALL when capacity < n (the first capacity are copied). */
int dvs_frames_load(const char *bundle_dir, dvs_frame *frames, size_t capacity, size_t *n_frames);
/* CameraTrajectory(frames, scene config) (include/dvs/trajectory.hpp:88-92);
 * DVS_ERR_INVALID for non-increasing or non-finite times, non-rigid poses,
 * invalid lighting or mount transforms. */
int dvs_trajectory_create(const dvs_frame *frames, size_t n_frames, const dvs_scene_config *scene,
                          dvs_trajectory **out);
int dvs_trajectory_destroy(dvs_trajectory *trajectory);
int dvs_trajectory_range(const dvs_trajectory *trajectory, float *start_time, float *end_time);
/* CameraTrajectory::evaluate(t) as an OpticalState (include/dvs/raycast.hpp:17-22);
 * orientation9 (row-major camera-to-world) may be NULL. */
int dvs_trajectory_evaluate(const dvs_trajectory *trajectory, float time, dvs_optical_state *state,
                            float *orientation9);

#ifdef __cplusplus
}
#endif
#endif /* DVS_GB300_H */
