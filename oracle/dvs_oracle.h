/*
 * CPU oracle for the DVS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C, the reference algorithm of
 * BugBubbles/DvsRender4DeepSpace for the event-camera hot path so that the
 * CUDA implementation can be checked against it.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load it; the product path never
 * does.
 *
 * The same source is compiled twice:
 *   liboracle_f32.so  -- the reference's own arithmetic: FP32 rays, triangle
 *                        test and Hapke, FP64 radiance sums, cos^4 and circuit.
 *                        Its sampler evaluates Hapke in the identity form of
 *                        the CUDA kernels (exact trigonometric identities,
 *                        see dvs_oracle.c); oracle_set_hapke_form(0) selects
 *                        the reference's own operation order.
 *   liboracle_f64.so  -- the same model with FP64 rays, geometry and Hapke
 *                        in the reference's order (the "FP64 oracle" used
 *                        for error reports).
 * Both are compiled with -ffp-contract=off so x86 and Arm give the same bits.
 *
 * Pinning: the circuit, Hapke, BVH build and FIFO readout are compared with
 * the reference's own host-compilable code (oracle/_ref, built from the
 * reference sources by oracle/Makefile) through golden fixtures in
 * tests/golden/, and the whole path against the known answers of the
 * reference tests (tests/test_sensor.cu, tests/test_render.cu,
 * tests/test_writer.cpp).
 *
 * Every function cites the reference file:line it follows.
 */
#ifndef DVS_ORACLE_H
#define DVS_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry records use float storage in both variants (the reference scene
 * is float3 vertex data, include/dvs/scene_types.hpp:129-150). */
typedef struct { float x, y, z; } of3;

/* BVHNode<float3> (include/dvs/scene_types.hpp:144-150): 40 bytes. */
typedef struct {
  of3 bmin, bmax;
  int32_t left, right, start, count;
} obvh_node;

/* HapkeConfig field order (include/dvs/scene_types.hpp:204-214). */
typedef struct {
  float b, c, hS, hC, thetap, w, B_S0, B_C0, phi;
} ohapke;

/* OpticalState (include/dvs/optical_sensor.hpp:148-152) without the CUDA
 * float4 alignment padding; quaternion is (x,y,z,w). */
typedef struct {
  of3 position, velocity, light, light_rate;
  float rotation[4];
  float intensity, intensity_rate;
} ostate;

typedef struct { ostate start, end; double t0, t1; } ointerval;

/* OpticalScene (include/dvs/optical_sensor.hpp:138-146). */
typedef struct {
  const obvh_node *nodes;
  const of3 *vertices, *normals;
  const uint32_t *indices;    /* 3 per triangle, BVH (leaf) order */
  const float *albedos;       /* per vertex, or NULL */
  int root, width, height, samples;
  float fx, fy, cx, cy;
  ohapke hapke;
  int32_t watertight;         /* 0: Moller-Trumbore (reference); 1: watertight test of the
                                 precision geometry (Woop et al. 2013) */
} oscene;

/* PixelParameters / PixelState (include/dvs/pixel_model.hpp:7-16). */
typedef struct {
  double threshold_pos, threshold_neg, charge_scale, refractory_time;
  double reference_leak, reset_noise_std;
} opixel_params;

typedef struct {
  double receptor_log, reference_log, refractory_until;
  double threshold_pos, threshold_neg;
  int32_t reset_pending;
} opixel_state;

/* PhotoParameters (include/dvs/optical_sensor.hpp:154-158). */
typedef struct {
  double electrons_per_radiance, dark_electrons, integration_step;
  int32_t shot_noise;
} ophoto;

/* PhysicConfig field order (include/dvs/scene_types.hpp:179-194). */
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
} ophysic;

/* Internal double-time event (include/dvs/dvs_base.hpp:9-18), unpacked. */
typedef struct {
  double timestamp;
  int16_t x, y;
  int8_t polarity;
  float depth;
} oevent;

/* ---- building blocks ---------------------------------------------------- */
double oracle_pi_f32(void);
int oracle_is_fp64(void);
float oracle_hapke_reflectance(float cosi, float cose, float cosg, float albedo, const ohapke *p);
float oracle_hapke_directional(const float *normal, const float *light, const float *view,
                               float albedo, const ohapke *p);
/* The Hapke form of the sampler: 1 = identity form (the CUDA kernels'
 * arithmetic; FP32 default), 0 = the reference's operation order (FP64
 * default).  oracle_hapke_reflectance/_directional always use form 0. */
void oracle_set_hapke_form(int form);
int oracle_hapke_form(void);
double oracle_hapke_reflectance_form(int form, double cosi, double cose, double cosg, double albedo,
                                     const ohapke *p);
double oracle_receptor_log_at(double u, double rate, double dt, double charge);
/* advance_pixel with a normal() draw that returns 0 (deterministic reset). */
int oracle_advance_pixel(opixel_state *s, const opixel_params *p, double rate, double t0, double t1,
                         double *event_t, int32_t *event_p, int capacity);
void oracle_derive_parameters(const ophysic *c, int physic_effects, opixel_params *p, ophoto *photo);
void oracle_optical_state_at(const ointerval *iv, double t, ostate *out);
/* Nearest hit through the binary BVH: returns hit (1), miss (0), overflow (-1). */
int oracle_trace_nearest(const oscene *s, const float *origin, const float *dir,
                         int *tri, float *t, float *u, float *v);
int oracle_trace_shadow(const oscene *s, const float *origin, const float *dir, int self_tri);
void oracle_shadow_origin(const oscene *s, int tri, float u, float v, const float *light, float *out);
void oracle_sample_pixel(const oscene *s, int pixel, const ostate *pose,
                         double *radiance, float *depth, int *valid);
/* Whole image at one pose; nthreads<=0 uses all OpenMP threads. */
void oracle_render(const oscene *s, const ostate *pose, double *radiance, float *depth,
                   int *valid, int nthreads);
/* Counted variant for timing: also returns primary and shadow rays traced. */
void oracle_render_pixels(const oscene *s, const ostate *pose, const int32_t *pixels, int n,
                          double *radiance, float *depth, int nthreads,
                          uint64_t *primary_rays, uint64_t *shadow_rays);

/* BVH build (src/bvh/build.cpp:27-76,126-187; src/bvh/bining.cpp:9-182).
 * indices (3 per triangle) are reordered in place to leaf order.
 * nodes must hold 2*n_triangles entries.  Returns the root index or -1. */
int oracle_bvh_build(int max_leaf_size, const float *vertices, int n_vertices,
                     uint32_t *indices, int n_triangles, obvh_node *nodes, int *n_nodes);
/* BVHBuilder::validate (src/bvh/build.cpp:188-242): 0 ok, -1 bad. */
int oracle_bvh_validate(const obvh_node *nodes, int n_nodes, int root);

/* ---- event readout FIFO (src/event_readout.cpp:6-34) -------------------- */
typedef struct oreadout oreadout;
oreadout *oracle_readout_create(double bandwidth, double latency, size_t capacity);
void oracle_readout_destroy(oreadout *r);
/* Sorts and queues events, then returns those ready at `now` (count in *n_ready). */
int oracle_readout_submit(oreadout *r, const oevent *events, size_t n, double now,
                          oevent *ready, size_t ready_cap, size_t *n_ready);
int oracle_readout_drain(oreadout *r, oevent *ready, size_t ready_cap, size_t *n_ready);
size_t oracle_readout_dropped(const oreadout *r);
size_t oracle_readout_peak(const oreadout *r);

/* ---- the event sensor (src/cuda/event_sensor.cu:18-60,244-305) ---------- */
typedef struct osensor osensor;
/* Deterministic physics only: threshold_std, shot noise and reset noise must
 * be off (the reference draws them from cuRAND, which has no CPU form). */
osensor *oracle_sensor_create(const oscene *scene, const ophysic *config, int physic_effects,
                              int aer_delay);
void oracle_sensor_destroy(osensor *s);
int oracle_sensor_initialize(osensor *s, const ostate *pose, double t, int nthreads);
/* Returns 0 ok, 1 capacity, 2 optical, 3 invalid argument, 6 output too small. */
int oracle_sensor_process(osensor *s, const ointerval *ivs, int n, oevent *out, size_t cap,
                          size_t *n_out, int nthreads);
int oracle_sensor_drain(osensor *s, oevent *out, size_t cap, size_t *n_out);
void oracle_sensor_states(const osensor *s, opixel_state *out);
size_t oracle_sensor_dropped(const osensor *s);
uint64_t oracle_sensor_rays(const osensor *s, int shadow);

/* ---- margin classification (no reference counterpart) -------------------
 * The accuracy statement exempts two classes from exact agreement, and these
 * calls name them instead of tolerating a fraction of differences:
 *   optical margin: a sub-ray whose outcome jumps when its image-plane
 *     direction moves by +-eta in x or y (eta several times the FP32 error of
 *     a ray direction): hit status, hit distance beyond 1e-3 (silhouette) or
 *     radiance term beyond 1e-3 (shadow / terminator boundary);
 *   circuit margin: a pixel whose polarity sequence changes when both
 *     thresholds move by +shift or by -shift (a log-intensity margin below
 *     shift at some crossing or near-crossing).
 *   conditioning (renders only): a pixel whose radiance or depth moves by
 *     more than the tolerance (1e-5) when all its sub-rays move by
 *     +-eta_c in x or y, eta_c (default 4 * 2^-24) about the FP32 error of a
 *     ray direction: no float ray fixes its value to the tolerance;
 *   crack (Moller-Trumbore scenes only): a primary hit within the FP32
 *     rounding bound of its barycentrics of an edge, where an FP32 test is not
 *     watertight and the ray can pass between two triangles;
 *   also optical margin: a lit sample at Hapke's azimuth singularity (cos psi
 *     evaluated in FP32 within the FP32 error of its cosines reaches -1), where
 *     the reference's FP32 formula yields NaN and drops the sample.
 * oracle_set_margin_eta sets eta for every later render and sensor call (0:
 * off, the default). */
void oracle_set_margin_eta(double eta);
/* eta_c and the relative change that makes a conditioning pixel (default
 * 4 * 2^-24 and 1e-5, the tolerance). */
void oracle_set_conditioning(double eta_c, double tolerance);
/* oracle_render_pixels with per-pixel flags (1: optical margin, 8:
 * conditioning, 16: crack); NaN radiance marks a traversal overflow. */
void oracle_render_pixels_margin(const oscene *s, const ostate *pose, const int32_t *pixels, int n,
                                 double *radiance, float *depth, uint8_t *margin, int nthreads);
/* Before initialize: track margins in this sensor (threshold_shift > 0). */
int oracle_sensor_set_margin(osensor *s, double threshold_shift);
/* Per pixel, row-major: 1 optical margin at a cell sample, 2 circuit margin,
 * 4 optical margin of an event-time depth sample, 16 crack at a cell sample. */
void oracle_sensor_margins(const osensor *s, uint8_t *out);

#ifdef __cplusplus
}
#endif
#endif
