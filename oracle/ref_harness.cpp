// extern "C" entry points over the REFERENCE's own host-compilable hot-path
// code, compiled from the reference sources by oracle/Makefile into
// oracle/_ref/libdvsref.so.  Test infrastructure only: it pins the oracle
// restatement (dvs_oracle.c) and generates the golden fixtures under
// tests/golden/.  Nothing here is product code and nothing here is shipped.
//
// Reference functions wrapped (paths within the reference project):
//   include/dvs/pixel_model.hpp:18-102   receptor_log_at, advance_pixel
//   include/dvs/hapke.hpp:131-172        hapke_reflectance, directional, invert_hapke_if
//   src/event_readout.cpp:6-34           EventReadout::submit / drain
//   src/bvh/build.cpp:27-242             BVHBuilder::build / validate
#include <cmath>
// nvcc host passes make isfinite visible globally; g++ needs the declaration.
using std::isfinite;
#include "dvs/pixel_model.hpp"
#include "dvs/hapke.hpp"
#include "dvs/event_sensor.hpp"
#include "bvh/build.h"
#include <cstring>
#include <vector>

namespace {
struct ZeroRng {
  double normal() { return 0; }  // tests/test_sensor.cu:10
};
}  // namespace

extern "C" {

double ref_receptor_log_at(double u, double rate, double dt, double charge) {
  return dvs::receptor_log_at(u, rate, dt, charge);
}

// state: receptor_log, reference_log, refractory_until, threshold_pos, threshold_neg, reset_pending
// params: threshold_pos, threshold_neg, charge_scale, refractory_time, reference_leak, reset_noise_std
int ref_advance_pixel(double *state, int *reset_pending, const double *params, double rate, double t0,
                      double t1, double *event_t, int *event_p, int capacity) {
  dvs::PixelState s;
  s.receptor_log = state[0]; s.reference_log = state[1]; s.refractory_until = state[2];
  s.threshold_pos = state[3]; s.threshold_neg = state[4]; s.reset_pending = *reset_pending != 0;
  dvs::PixelParameters p;
  p.threshold_pos = params[0]; p.threshold_neg = params[1]; p.charge_scale = params[2];
  p.refractory_time = params[3]; p.reference_leak = params[4]; p.reset_noise_std = params[5];
  std::vector<dvs::PixelEvent> out(capacity > 0 ? capacity : 1);
  ZeroRng rng;
  int n = dvs::advance_pixel(s, p, rate, t0, t1, out.data(), capacity, rng);
  for (int i = 0; i < n; ++i) { event_t[i] = out[i].time; event_p[i] = out[i].polarity; }
  state[0] = s.receptor_log; state[1] = s.reference_log; state[2] = s.refractory_until;
  state[3] = s.threshold_pos; state[4] = s.threshold_neg; *reset_pending = s.reset_pending;
  return n;
}

static dvs::HapkeConfig hapke_from(const float *h) {
  dvs::HapkeConfig p;
  p.b = h[0]; p.c = h[1]; p.hS = h[2]; p.hC = h[3]; p.thetap = h[4];
  p.w = h[5]; p.B_S0 = h[6]; p.B_C0 = h[7]; p.phi = h[8];
  return p;
}

float ref_hapke_reflectance(float cosi, float cose, float cosg, float albedo, const float *h) {
  return dvs::hapke_reflectance(cosi, cose, cosg, albedo, hapke_from(h));
}

float ref_hapke_directional(const float *n, const float *l, const float *v, float albedo, const float *h) {
  return dvs::hapke_directional_reflectance(make_float3(n[0], n[1], n[2]), make_float3(l[0], l[1], l[2]),
                                            make_float3(v[0], v[1], v[2]), albedo, hapke_from(h));
}

float ref_invert_hapke_if(float inc, float emi, float phase, float target, const float *h) {
  return dvs::invert_hapke_if(inc, emi, phase, target, hapke_from(h));
}

// nodes_out: 10 x 4-byte words per node (BVHNode<float3>, 40 bytes); capacity 2*n_triangles.
int ref_bvh_build(int max_leaf, const float *vertices, int n_vertices, unsigned *indices, int n_triangles,
                  void *nodes_out, int *n_nodes) {
  std::vector<float3> v(n_vertices);
  for (int i = 0; i < n_vertices; ++i) v[i] = make_float3(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
  std::vector<uint3> t(n_triangles);
  for (int i = 0; i < n_triangles; ++i) t[i] = make_uint3(indices[3 * i], indices[3 * i + 1], indices[3 * i + 2]);
  dvs::BVHBuildParams params;
  params.max_leaf_size = max_leaf;
  std::vector<dvs::BVHNode<float3>> nodes;
  int root = dvs::BVHBuilder::build(params, nodes, t, v);
  static_assert(sizeof(dvs::BVHNode<float3>) == 40, "node layout");
  std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(dvs::BVHNode<float3>));
  *n_nodes = static_cast<int>(nodes.size());
  for (int i = 0; i < n_triangles; ++i) { indices[3 * i] = t[i].x; indices[3 * i + 1] = t[i].y; indices[3 * i + 2] = t[i].z; }
  return root;
}

// Packed 17-byte events (include/dvs/dvs_base.hpp:9-18).
void *ref_readout_create(double bandwidth, double latency, size_t capacity) {
  return new dvs::EventReadout(bandwidth, latency, capacity);
}
void ref_readout_destroy(void *r) { delete static_cast<dvs::EventReadout *>(r); }
size_t ref_readout_submit(void *r, const void *events, size_t n, double now, void *ready, size_t cap) {
  static_assert(sizeof(dvs::Event) == 17, "event layout");
  std::vector<dvs::Event> in(n), out;
  if (n) std::memcpy(in.data(), events, n * sizeof(dvs::Event));
  static_cast<dvs::EventReadout *>(r)->submit(std::move(in), now, out);
  size_t m = out.size() < cap ? out.size() : cap;
  if (m) std::memcpy(ready, out.data(), m * sizeof(dvs::Event));
  return out.size();
}
size_t ref_readout_drain(void *r, void *ready, size_t cap) {
  std::vector<dvs::Event> out;
  static_cast<dvs::EventReadout *>(r)->drain(out);
  size_t m = out.size() < cap ? out.size() : cap;
  if (m) std::memcpy(ready, out.data(), m * sizeof(dvs::Event));
  return out.size();
}
size_t ref_readout_dropped(void *r) { return static_cast<dvs::EventReadout *>(r)->dropped(); }
size_t ref_readout_peak(void *r) { return static_cast<dvs::EventReadout *>(r)->peak_queue(); }

}  // extern "C"
