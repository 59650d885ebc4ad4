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
//     walk the 4-wide BVH together (warp-uniform control flow, node and
//     triangle records fetched once per warp as 16-byte broadcast loads); each
//     lane keeps its own closest hit.  The traversal stack is warp-uniform and
//     lives in registers distributed across the lanes.
//   * circuit: one thread per pixel streams the per-cell radiance of a chunk
//     and integrates the pixel circuit in FP64 (pixel_model.hpp semantics).
//   * emit_events: warp prefix-sum compaction of the per-pixel event slabs.
//   * event_depth: depth re-trace at each event time (event_sensor.cu:51-59).
#include <cstdint>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "kernels.h"

namespace dvsgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr float kRayEps = 1e-6f;          // include/helper_math.hpp:12
constexpr float kPi = 3.14159265358979323846f;  // include/dvs/math_types.hpp:37
__device__ __forceinline__ float kInf() { return __int_as_float(0x7f800000); }

// ---- float3 algebra (include/helper_math.hpp:18-77) -------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize(float3 v) {
  float len = sqrtf(dot(v, v));
  if (len > 0.0f) return v / len;
  return f3(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// ---- Hapke (include/dvs/hapke.hpp:14-157), FP32 --------------------------------
__device__ __forceinline__ float safe_tan(float x) {
  return tanf(clampf(x, -kPi / 2.0f + 1e-6f, kPi / 2.0f - 1e-6f));
}
__device__ __forceinline__ float safe_acos(float x) { return acosf(clampf(x, -1.0f, 1.0f)); }
__device__ __forceinline__ float hg_double_lobe(float cosg, float b, float c) {
  const float one_minus_bb = 1.0f - b * b;
  const float term1 = ((1.0f + c) * 0.5f) * one_minus_bb / powf(1.0f - 2.0f * b * cosg + b * b, 1.5f);
  const float term2 = ((1.0f - c) * 0.5f) * one_minus_bb / powf(1.0f + 2.0f * b * cosg + b * b, 1.5f);
  return term1 + term2;
}
__device__ __forceinline__ float b_s(float tg, float h) {
  if (h <= 0.0f) return tg <= 0.0f ? 1.0f : 0.0f;
  return 1.0f / (1.0f + tg / h);
}
__device__ __forceinline__ float b_c(float tg, float h) {
  if (h <= 0.0f) return tg <= 0.0f ? 1.0f : 0.0f;
  const float T = tg / h;
  if (T < 1e-8f) return 1.0f;
  return (1.0f + (1.0f - expf(-T)) / T) / (2.0f * (1.0f + T) * (1.0f + T));
}
__device__ __forceinline__ float hfunc(float x, float w) {
  if (x <= 1e-8f) return 1.0f;
  const float root = sqrtf(fmaxf(0.0f, 1.0f - w));
  const float r0 = (1.0f - root) / (1.0f + root);
  const float term = r0 + (1.0f - 2.0f * r0 * x) * 0.5f * logf(1.0f + 1.0f / x);
  return 1.0f / (1.0f - w * x * term);
}
__device__ __forceinline__ float porosity_k(float phi) {
  if (phi <= 1e-8f) return 1.0f;
  const float p = 1.209f * powf(phi, 2.0f / 3.0f);
  return -logf(1.0f - p) / p;
}
__device__ __forceinline__ float chi_f(float thetap) {
  const float t = tanf(thetap);
  return 1.0f / sqrtf(1.0f + kPi * t * t);
}
__device__ __forceinline__ float e1_f(float thetap, float cosy, float siny) {
  const float s = fmaxf(siny, 1e-6f);
  return expf((-2.0f / kPi) * (1.0f / tanf(thetap)) * cosy / s);
}
__device__ __forceinline__ float e2_f(float thetap, float cosy, float siny) {
  const float s = fmaxf(siny, 1e-6f);
  const float v = (1.0f / tanf(thetap)) * cosy / s;
  return expf((-1.0f / kPi) * v * v);
}
__device__ __forceinline__ float eta_f(float thetap, float cosy, float siny) {
  const float ch = chi_f(thetap);
  const float e1 = e1_f(thetap, cosy, siny);
  const float e2 = e2_f(thetap, cosy, siny);
  return ch * (cosy + siny * tanf(thetap) * e2 / (2.0f - e1));
}
__device__ __forceinline__ float f_psi(float psi) { return expf(-2.0f * tanf(psi * 0.5f)); }

__device__ float hapke_reflectance(float cosi, float cose, float cosg, float albedo, const dvs_hapke &p) {
  if (cosi <= 0 || cose <= 0) return 0;
  cosi = clampf(cosi, 0, 1);
  cose = clampf(cose, 0, 1);
  cosg = clampf(cosg, -1, 1);
  const float sini = sqrtf(fmaxf(0, 1 - cosi * cosi)), sine = sqrtf(fmaxf(0, 1 - cose * cose));
  const float tg = safe_tan(safe_acos(cosg) * 0.5f);
  const float psi = safe_acos((cosg - cosi * cose) / (sini * sine + 1e-6f));
  const float p_g = hg_double_lobe(cosg, p.b, p.c);
  const float BS = b_s(tg, p.hS);
  const float BC = b_c(tg, p.hC);
  const float K = porosity_k(p.phi);
  float mu0, mue, S;
  const float thetap = p.thetap;
  if (thetap <= 1e-8f) {
    mu0 = cosi; mue = cose; S = 1.0f;
  } else {
    const float ch = chi_f(thetap);
    const float tan_thetap = tanf(thetap);
    const float sh = sinf(psi * 0.5f);
    const float s2 = sh * sh;
    const float e2e = e2_f(thetap, cose, sine), e2i = e2_f(thetap, cosi, sini);
    const float e1e = e1_f(thetap, cose, sine), e1i = e1_f(thetap, cosi, sini);
    const float eta_e = eta_f(thetap, cose, sine), eta_i = eta_f(thetap, cosi, sini);
    const float fp = f_psi(psi);
    if (cosi >= cose) {
      mu0 = ch * (cosi + sini * tan_thetap * (cosf(psi) * e2e + s2 * e2i) / (2.0f - e1e - (psi / kPi) * e1i));
      mue = ch * (cose + sine * tan_thetap * (e2e - s2 * e2i) / (2.0f - e1e - (psi / kPi) * e1i));
      S = mue / eta_e * cosi / eta_i * ch / (1.0f - fp + fp * ch * (cosi / eta_i));
    } else {
      mu0 = ch * (cosi + sini * tan_thetap * (e2i - s2 * e2e) / (2.0f - e1i - (psi / kPi) * e1e));
      mue = ch * (cose + sine * tan_thetap * (cosf(psi) * e2i + s2 * e2e) / (2.0f - e1i - (psi / kPi) * e1e));
      S = mue / eta_e * cosi / eta_i * ch / (1.0f - fp + fp * ch * (cose / eta_e));
    }
  }
  const float M = hfunc(mu0 / K, albedo) * hfunc(mue / K, albedo) - 1.0f;
  const float LS = mu0 / (mu0 + mue + 1e-6f);
  return (albedo / (4.0f * kPi)) * LS * K * (p_g * (1.0f + BS * p.B_S0) + M) * (1.0f + BC * p.B_C0) * S;
}

// ---- pose interpolation (include/dvs/device_optics.cuh:6-29) ---------------------
__device__ __forceinline__ float hermite(float a, float va, float b, float vb, float u, float dt) {
  float u2 = u * u, u3 = u2 * u;
  return a + (-2 * u3 + 3 * u2) * (b - a) + (u3 - 2 * u2 + u) * dt * va + (u3 - u2) * dt * vb;
}
__device__ __forceinline__ float3 ld3(const dvs_float3 &v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 hermite3(const dvs_float3 &a, const dvs_float3 &va, const dvs_float3 &b,
                                           const dvs_float3 &vb, float u, float dt) {
  return f3(hermite(a.x, va.x, b.x, vb.x, u, dt), hermite(a.y, va.y, b.y, vb.y, u, dt),
            hermite(a.z, va.z, b.z, vb.z, u, dt));
}
// optical_state_at reduced to what the ray generator needs.  The quaternion
// is renormalized with a correctly rounded 1/sqrt (the reference's rsqrtf is
// an approximation the CPU oracle cannot reproduce).
__device__ CellPose pose_at(const dvs_optical_interval &iv, double t) {
  float dt = iv.t1 - iv.t0, u = dt > 0 ? fmin(1.0, fmax(0.0, (t - iv.t0) / dt)) : 0;
  float3 pos = hermite3(iv.start.position, iv.start.velocity, iv.end.position, iv.end.velocity, u, dt);
  float3 light = hermite3(iv.start.light, iv.start.light_rate, iv.end.light, iv.end.light_rate, u, dt);
  float intensity = fmaxf(0, hermite(iv.start.intensity, iv.start.intensity_rate, iv.end.intensity,
                                     iv.end.intensity_rate, u, dt));
  float4 a = make_float4(iv.start.rotation.x, iv.start.rotation.y, iv.start.rotation.z, iv.start.rotation.w);
  float4 b = make_float4(iv.end.rotation.x, iv.end.rotation.y, iv.end.rotation.z, iv.end.rotation.w);
  float d = a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
  if (d < 0) { b = make_float4(-b.x, -b.y, -b.z, -b.w); d = -d; }
  float wa = 1 - u, wb = u;
  if (d < .9995f) {
    float angle = acosf(fminf(1, d)), inv = 1 / sinf(angle);
    wa = sinf((1 - u) * angle) * inv;
    wb = sinf(u * angle) * inv;
  }
  float4 q = make_float4(wa * a.x + wb * b.x, wa * a.y + wb * b.y, wa * a.z + wb * b.z, wa * a.w + wb * b.w);
  float norm = 1.0f / sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  float3 ln = normalize(light);  // sample_pixel normalizes pose.light (device_optics.cuh:75)
  CellPose out;
  out.px = pos.x; out.py = pos.y; out.pz = pos.z; out.intensity = intensity;
  out.qx = q.x * norm; out.qy = q.y * norm; out.qz = q.z * norm; out.qw = q.w * norm;
  out.lx = ln.x; out.ly = ln.y; out.lz = ln.z; out.pad = 0;
  return out;
}
__device__ __forceinline__ float3 rotate_ray(const CellPose &q, float3 v) {
  float3 qv = f3(q.qx, q.qy, q.qz);
  float3 c = 2 * cross(qv, v);
  return v + q.qw * c + cross(qv, c);
}

// ---- traversal -------------------------------------------------------------------
__device__ __forceinline__ float3 inverse_direction(float3 d) {  // device_ray.hpp:6-12
  float3 inv;
  inv.x = 1.0f / (fabsf(d.x) > 1e-20f ? d.x : copysignf(1e-20f, d.x));
  inv.y = 1.0f / (fabsf(d.y) > 1e-20f ? d.y : copysignf(1e-20f, d.y));
  inv.z = 1.0f / (fabsf(d.z) > 1e-20f ? d.z : copysignf(1e-20f, d.z));
  return inv;
}

// Moller-Trumbore with precomputed edges (device_ray.hpp:54-80).
__device__ __forceinline__ bool intersect_tri(float3 ray, float3 o, float3 v0, float3 e1, float3 e2, float &t,
                                              float &u, float &v) {
  const float3 pvec = cross(ray, e2);
  const float det = dot(e1, pvec);
  if (fabsf(det) < kRayEps) return false;
  const float inv_det = 1.0f / det;
  const float3 tvec = o - v0;
  u = dot(tvec, pvec) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const float3 qvec = cross(tvec, e1);
  v = dot(ray, qvec) * inv_det;
  if (v < 0.0f || (u + v) > 1.0f) return false;
  t = dot(e2, qvec) * inv_det;
  if (t <= kRayEps) return false;
  return true;
}

struct NodeBoxes {
  float4 lx, hx, ly, hy, lz, hz;
  int4 child, count;
};
__device__ __forceinline__ NodeBoxes load_node(const Bvh4Node *n) {
  const float4 *p = reinterpret_cast<const float4 *>(n);
  NodeBoxes b;
  b.lx = __ldg(p + 0); b.hx = __ldg(p + 1);
  b.ly = __ldg(p + 2); b.hy = __ldg(p + 3);
  b.lz = __ldg(p + 4); b.hz = __ldg(p + 5);
  b.child = __ldg(reinterpret_cast<const int4 *>(p + 6));
  b.count = __ldg(reinterpret_cast<const int4 *>(p + 7));
  return b;
}
// Slab test of one child (device_ray.hpp:21-29 form).
__device__ __forceinline__ bool slab(float lx, float hx, float ly, float hy, float lz, float hz, float3 o,
                                     float3 idir, float t_min, float t_max, float &tnear) {
  float tx0 = (lx - o.x) * idir.x, tx1 = (hx - o.x) * idir.x;
  float ty0 = (ly - o.y) * idir.y, ty1 = (hy - o.y) * idir.y;
  float tz0 = (lz - o.z) * idir.z, tz1 = (hz - o.z) * idir.z;
  float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  tmin = fmaxf(t_min, tmin);
  tmax = fminf(t_max, tmax);
  tnear = tmin;
  return tmax >= tmin;
}
__device__ __forceinline__ unsigned child_mask(const NodeBoxes &b, float3 o, float3 idir, float t_min, float t_max,
                                               float tn[4]) {
  unsigned m = 0;
  if (b.count.x >= 0 && slab(b.lx.x, b.hx.x, b.ly.x, b.hy.x, b.lz.x, b.hz.x, o, idir, t_min, t_max, tn[0])) m |= 1;
  if (b.count.y >= 0 && slab(b.lx.y, b.hx.y, b.ly.y, b.hy.y, b.lz.y, b.hz.y, o, idir, t_min, t_max, tn[1])) m |= 2;
  if (b.count.z >= 0 && slab(b.lx.z, b.hx.z, b.ly.z, b.hy.z, b.lz.z, b.hz.z, o, idir, t_min, t_max, tn[2])) m |= 4;
  if (b.count.w >= 0 && slab(b.lx.w, b.hx.w, b.ly.w, b.hy.w, b.lz.w, b.hz.w, o, idir, t_min, t_max, tn[3])) m |= 8;
  return m;
}
__device__ __forceinline__ int comp(const int4 &v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }
// Stack entry: inner node index (>= 0) or ~(first_triangle << 3 | count - 1).
__device__ __forceinline__ int encode_child(const NodeBoxes &b, int c) {
  const int cnt = comp(b.count, c), ch = comp(b.child, c);
  return cnt > 0 ? ~((ch << 3) | (cnt - 1)) : ch;
}

// Warp-uniform stack: slot k lives in lane k%32 of register bank k/32; each
// lane keeps its own entry distance for the slot in tdist[k] (local memory,
// lane-interleaved, so one uniform slot index is one coalesced access).
struct WarpStack {
  int b0, b1, b2;
  int sp;
  __device__ __forceinline__ void init() { b0 = b1 = b2 = 0; sp = 0; }
  __device__ __forceinline__ bool push(int lane, int value, float *tdist, float t) {
    if (sp >= kStackSlots) return false;
    if (lane == (sp & 31)) {
      const int bank = sp >> 5;
      if (bank == 0) b0 = value; else if (bank == 1) b1 = value; else b2 = value;
    }
    tdist[sp] = t;
    ++sp;
    return true;
  }
  __device__ __forceinline__ int pop(float *tdist, float &t) {
    --sp;
    const int bank = sp >> 5;
    const int reg = bank == 0 ? b0 : (bank == 1 ? b1 : b2);
    t = tdist[sp];
    return __shfl_sync(kFull, reg, sp & 31);
  }
};

struct HitRecord {
  int hit;  // 1 hit, 0 miss, -1 stack overflow (device_ray.hpp:152)
  int tri;
  float t, u, v;
};

// Nearest hit for the 32 rays of a warp (trace_nearest, device_ray.hpp:136-158).
// All lanes must call converged; inactive lanes never hit.
__device__ HitRecord trace_nearest_packet(const SceneView &S, float3 o, float3 d, bool active, float *tdist) {
  const int lane = threadIdx.x & 31;
  const float3 idir = inverse_direction(d);
  float closest = active ? 1e30f : -1.0f;
  HitRecord h{0, -1, 0.f, 0.f, 0.f};
  WarpStack st;
  st.init();
  int entry = 0;  // root: node 0
  float entry_t = active ? 0.0f : kInf();
  bool overflow = false;
  while (true) {
    if (__any_sync(kFull, entry_t <= closest)) {
      if (entry >= 0) {
        const NodeBoxes nb = load_node(S.nodes + entry);
        float tn[4] = {kInf(), kInf(), kInf(), kInf()};
        const unsigned m = child_mask(nb, o, idir, kRayEps, closest, tn);
        const unsigned any = __reduce_or_sync(kFull, m);
        if (any) {
          const int leader = __ffs(__ballot_sync(kFull, m != 0)) - 1;
          float key[4];
          int ids[4];
          int n = 0;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float k = __shfl_sync(kFull, (m >> c) & 1 ? tn[c] : kInf(), leader);
            if ((any >> c) & 1) { key[n] = k; ids[n] = c; ++n; }
          }
          // insertion sort, nearest first (uniform)
          for (int i = 1; i < n; ++i)
            for (int j = i; j > 0 && key[j] < key[j - 1]; --j) {
              float tk = key[j]; key[j] = key[j - 1]; key[j - 1] = tk;
              int ti = ids[j]; ids[j] = ids[j - 1]; ids[j - 1] = ti;
            }
          for (int i = n - 1; i >= 1; --i) {
            const int c = ids[i];
            const float mine = (m >> c) & 1 ? tn[c] : kInf();
            if (!st.push(lane, encode_child(nb, c), tdist, mine)) overflow = true;
          }
          const int c0 = ids[0];
          entry = encode_child(nb, c0);
          entry_t = (m >> c0) & 1 ? tn[c0] : kInf();
          if (overflow) break;
          continue;
        }
      } else {
        const int code = ~entry;
        const int first = code >> 3, count = (code & 7) + 1;
        const bool need = entry_t <= closest;  // this lane's own box test reached the leaf
        for (int i = 0; i < count; ++i) {
          const float4 *r = reinterpret_cast<const float4 *>(S.tris + first + i);
          const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
          float t, u, v;
          if (need && intersect_tri(d, o, f3(a.x, a.y, a.z), f3(a.w, b.x, b.y), f3(b.z, b.w, c.x), t, u, v) &&
              t < closest) {
            closest = t;
            h.hit = 1; h.tri = first + i; h.t = t; h.u = u; h.v = v;
          }
        }
      }
    }
    if (st.sp == 0) break;
    entry = st.pop(tdist, entry_t);
  }
  if (overflow) h.hit = -1;
  return h;
}

// Any hit toward the light (trace_shadow_ray_any_hit, device_ray.hpp:81-135):
// skips the camera-hit triangle, t in (kRayEps, 1e30); overflow counts as occluded.
__device__ bool trace_shadow_packet(const SceneView &S, float3 o, float3 d, bool active, int self, float *tdist) {
  const int lane = threadIdx.x & 31;
  const float3 idir = inverse_direction(d);
  bool alive = active;
  bool occluded = false;
  WarpStack st;
  st.init();
  int entry = 0;
  float entry_t = alive ? 0.0f : kInf();
  const float t_max = 1e30f;
  while (true) {
    if (__any_sync(kFull, alive && entry_t <= t_max)) {
      if (entry >= 0) {
        const NodeBoxes nb = load_node(S.nodes + entry);
        float tn[4] = {kInf(), kInf(), kInf(), kInf()};
        const unsigned m = child_mask(nb, o, idir, kRayEps, alive ? t_max : -1.0f, tn);
        const unsigned any = __reduce_or_sync(kFull, m);
        if (any) {
          int first_c = -1;
          bool overflow = false;
#pragma unroll
          for (int c = 3; c >= 0; --c) {
            if (!((any >> c) & 1)) continue;
            if (first_c < 0) { first_c = c; continue; }
            if (!st.push(lane, encode_child(nb, first_c), tdist, (m >> first_c) & 1 ? tn[first_c] : kInf()))
              overflow = true;
            first_c = c;
          }
          if (overflow) {  // conservative: occluded (device_ray.hpp:119)
            occluded = occluded || alive;
            break;
          }
          entry = encode_child(nb, first_c);
          entry_t = (m >> first_c) & 1 ? tn[first_c] : kInf();
          continue;
        }
      } else {
        const int code = ~entry;
        const int first = code >> 3, count = (code & 7) + 1;
        const bool need = entry_t <= t_max;
        for (int i = 0; i < count; ++i) {
          const int id = first + i;
          const float4 *r = reinterpret_cast<const float4 *>(S.tris + id);
          const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
          float t, u, v;
          if (alive && need && id != self &&
              intersect_tri(d, o, f3(a.x, a.y, a.z), f3(a.w, b.x, b.y), f3(b.z, b.w, c.x), t, u, v) &&
              t > kRayEps && t < t_max) {
            occluded = true;
            alive = false;
          }
        }
        if (!__any_sync(kFull, alive)) break;
      }
    }
    if (st.sp == 0) break;
    entry = st.pop(tdist, entry_t);
  }
  return occluded;
}

// shadow_origin (device_optics.cuh:37-51) from the leaf-order triangle record.
__device__ float3 shadow_origin(const TriRecord &tr, float u, float v, float3 light) {
  float3 a = f3(tr.v0[0], tr.v0[1], tr.v0[2]), e1 = f3(tr.e1[0], tr.e1[1], tr.e1[2]),
         e2 = f3(tr.e2[0], tr.e2[1], tr.e2[2]);
  float3 point = a + u * e1 + v * e2, normal = normalize(cross(e1, e2));
  if (dot(normal, light) < 0) normal = -normal;
  constexpr float epsilon = 5.960464477539063e-8f, gamma = 8 * epsilon / (1 - 8 * epsilon);
  float3 error = f3(gamma * (fabsf(a.x) + fabsf(u * e1.x) + fabsf(v * e2.x)),
                    gamma * (fabsf(a.y) + fabsf(u * e1.y) + fabsf(v * e2.y)),
                    gamma * (fabsf(a.z) + fabsf(u * e1.z) + fabsf(v * e2.z)));
  float distance = fabsf(normal.x) * error.x + fabsf(normal.y) * error.y + fabsf(normal.z) * error.z + 1e-6f;
  float3 offset = normal * distance;
  point = point + offset;
  if (offset.x != 0) point.x = nextafterf(point.x, copysignf(kInf(), offset.x));
  if (offset.y != 0) point.y = nextafterf(point.y, copysignf(kInf(), offset.y));
  if (offset.z != 0) point.z = nextafterf(point.z, copysignf(kInf(), offset.z));
  return point;
}

struct PixelSample {
  double radiance;
  float depth;
  bool valid;
  unsigned primary, shadow;
};

// sample_pixel (device_optics.cuh:73-94) for one lane of a converged warp.
// depth_only skips shading (the event-time depth of event_sensor.cu:55).
template <bool kDepthOnly>
__device__ PixelSample sample_pixel_packet(const SceneView &S, int pixel, bool active, const CellPose &pose,
                                           float *tdist) {
  PixelSample out{0.0, -1.0f, true, 0u, 0u};
  double depth = 0;
  int valid_depth = 0;
  const float3 light = f3(pose.lx, pose.ly, pose.lz);
  const float3 origin = f3(pose.px, pose.py, pose.pz);
  const int ss = S.samples;
  const int px_i = pixel % S.width, py_i = pixel / S.width;
  for (int sy = 0; sy < ss; ++sy)
    for (int sx = 0; sx < ss; ++sx) {
      float px = (px_i + (sx + .5f) / ss - .5f - S.cx) / S.fx;
      float py = (py_i + (sy + .5f) / ss - .5f - S.cy) / S.fy;
      float3 ray = normalize(rotate_ray(pose, f3(px, -py, -1)));
      const HitRecord hit = trace_nearest_packet(S, origin, ray, active && out.valid, tdist);
      if (active && out.valid) ++out.primary;
      if (hit.hit < 0) out.valid = false;
      const bool hitp = active && out.valid && hit.hit == 1;
      bool lit = false;
      float3 normal = f3(0, 0, 0), sorigin = f3(0, 0, 0);
      float albedo = S.hapke.w;
      if (hitp) {
        depth += hit.t;
        ++valid_depth;
        if (!kDepthOnly) {
          const ShadeRecord *sr = S.shade + hit.tri;
          const float4 *q = reinterpret_cast<const float4 *>(sr);
          const float4 s0 = __ldg(q), s1 = __ldg(q + 1), s2 = __ldg(q + 2);
          const float w = 1 - hit.u - hit.v;
          normal = normalize(f3(s0.x, s0.y, s0.z) * w + f3(s1.x, s1.y, s1.z) * hit.u + f3(s2.x, s2.y, s2.z) * hit.v);
          lit = !(dot(normal, light) <= 0 || dot(normal, -ray) <= 0);
          if (lit) {
            const TriRecord tr = S.tris[hit.tri];
            sorigin = shadow_origin(tr, hit.u, hit.v, light);
            if (S.has_albedo) albedo = s0.w * w + s1.w * hit.u + s2.w * hit.v;
          }
        }
      }
      if (!kDepthOnly) {
        if (__any_sync(kFull, lit)) {
          if (lit) ++out.shadow;
          const bool occ = trace_shadow_packet(S, sorigin, light, lit, hit.tri, tdist);
          if (lit && !occ) {
            double cos4 = 1.0 / ((1.0 + px * px + py * py) * (1.0 + px * px + py * py));
            float n_h = 0;
            {  // hapke_directional_reflectance (hapke.hpp:153-157)
              float3 n = normalize(normal), l = normalize(light), v = normalize(-ray);
              n_h = hapke_reflectance(dot(n, l), dot(n, v), dot(l, v), albedo, S.hapke);
            }
            out.radiance += fmaxf(0, n_h * pose.intensity) * cos4;
          }
        }
      }
    }
  out.radiance /= ss * ss;
  out.depth = valid_depth ? float(depth / valid_depth) : -1.0f;
  return out;
}

__device__ __forceinline__ unsigned warp_sum(unsigned v) { return __reduce_add_sync(kFull, v); }

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

__global__ void cell_poses_kernel(const dvs_optical_interval *ivs, const Cell *cells, int n, CellPose *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const Cell cell = cells[c];
  out[c] = pose_at(ivs[cell.interval], (cell.t0 + cell.t1) * .5);
}

__global__ void __launch_bounds__(128) trace_cells_kernel(SceneView S, int n_pix, const CellPose *poses, int c0,
                                                          int nc, int cw_log2, double *radiance, float *depth_out,
                                                          unsigned long long *counters) {
  float tdist[kStackSlots];
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)(blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int cw = 1 << cw_log2, ppw = 32 >> cw_log2;
  const int n_groups = (nc + cw - 1) >> cw_log2;
  const long long pgroup = warp / n_groups;
  const int g = (int)(warp % n_groups);
  if (pgroup * ppw >= n_pix) return;  // warp-uniform
  const int rank = (int)(pgroup * ppw) + (lane >> cw_log2);
  const int cell = g * cw + (lane & (cw - 1));
  const bool active = rank < n_pix && cell < nc;
  const int pixel = active ? __ldg(S.pixel_of_rank + rank) : 0;
  const CellPose pose = poses[c0 + (active ? cell : 0)];
  const PixelSample s = sample_pixel_packet<false>(S, pixel, active, pose, tdist);
  if (active) {
    const size_t o = (size_t)cell * n_pix + rank;
    radiance[o] = s.valid ? s.radiance : __longlong_as_double(0x7ff8000000000000ll);
    if (depth_out) depth_out[o] = s.depth;
  }
  const unsigned prim = warp_sum(s.primary), shad = warp_sum(s.shadow);
  if (lane == 0 && counters) {
    atomicAdd(counters + kCntPrimary, (unsigned long long)prim);
    atomicAdd(counters + kCntShadow, (unsigned long long)shad);
  }
}

// ---- pixel circuit (include/dvs/pixel_model.hpp:18-102), FP64 ------------------------
__device__ __forceinline__ double receptor_log_at(double u, double rate, double dt, double charge) {
  if (dt <= 0) return u;
  rate = fmax(0.0, rate);
  double x = exp(u);
  if (rate == 0) return u - log1p(x * dt / charge);
  double a = exp(-rate * dt / charge), b = -expm1(-rate * dt / charge);
  return -log(a / x + b / rate);
}

struct PixelRegs {
  double receptor_log, reference_log, refractory_until, threshold_pos, threshold_neg;
  bool reset_pending;
};

// Returns events emitted, -1 at capacity, -2 when the loop stops making progress.
__device__ int advance_pixel(PixelRegs &s, const PixelParams &p, double rate, double t0, double t1, double *out_t,
                             int8_t *out_p, int capacity, curandStateXORWOW_t &rng) {
  if (t1 <= t0) return 0;
  int count = 0;
  double cursor = t0, u = s.receptor_log;
  int passes = 0;
  while (cursor < t1) {
    if (++passes > 4096) return -2;  // bounded: see kErrStalled
    if (cursor < s.refractory_until) {
      double end = fmin(t1, s.refractory_until);
      u = receptor_log_at(u, rate, end - cursor, p.charge_scale);
      cursor = end;
      s.reference_log = u;
      if (cursor < t1 || cursor == s.refractory_until) {
        if (cursor >= s.refractory_until && s.reset_pending) {
          if (p.reset_noise_std > 0) s.reference_log += p.reset_noise_std * curand_normal_double(&rng);
          s.reset_pending = false;
        }
      }
      if (cursor >= t1) break;
    } else if (s.reset_pending) {
      if (p.reset_noise_std > 0) s.reference_log += p.reset_noise_std * curand_normal_double(&rng);
      s.reset_pending = false;
    }
    double remaining = t1 - cursor;
    double c0 = u - s.reference_log;
    double boundary = remaining;
    double x = exp(u), target = rate + p.charge_scale * p.reference_leak;
    if (p.reference_leak > 0 && x > target && target > rate) {
      double extremum;
      if (rate > 0) extremum = -p.charge_scale / rate * log((1.0 / target - 1.0 / rate) / (1.0 / x - 1.0 / rate));
      else extremum = p.charge_scale * (1.0 / target - 1.0 / x);
      if (extremum > 1e-15 && extremum < boundary) boundary = extremum;
    }
    double ub = receptor_log_at(u, rate, boundary, p.charge_scale);
    double cb = ub - s.reference_log + p.reference_leak * boundary;
    int polarity = -1;
    double level = 0;
    if (c0 >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (c0 <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    else if (cb >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (cb <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    if (polarity < 0) {
      u = ub;
      s.reference_log -= p.reference_leak * boundary;
      cursor += boundary;
      continue;
    }
    if (count == capacity) return -1;
    double lo = 0, hi = boundary;
    if (c0 >= s.threshold_pos || c0 <= -s.threshold_neg) hi = 0;
    else if (p.reference_leak == 0) {
      double target_inverse = exp(-(s.reference_log + level));
      double initial_inverse = exp(-u);
      if (rate > 0) {
        double stationary_inverse = 1.0 / rate;
        hi = -p.charge_scale / rate * log1p((target_inverse - initial_inverse) / (initial_inverse - stationary_inverse));
      } else hi = p.charge_scale * (target_inverse - initial_inverse);
      hi = fmin(boundary, fmax(0.0, hi));
    } else
      for (int j = 0; j < 48; ++j) {
        double mid = (lo + hi) * .5;
        double c = receptor_log_at(u, rate, mid, p.charge_scale) - s.reference_log + p.reference_leak * mid;
        if (polarity ? c >= level : c <= level) hi = mid; else lo = mid;
      }
    u = receptor_log_at(u, rate, hi, p.charge_scale);
    cursor += hi;
    out_t[count] = cursor;
    out_p[count] = (int8_t)polarity;
    ++count;
    s.reference_log = u;
    s.refractory_until = cursor + p.refractory_time;
    s.reset_pending = true;
  }
  s.receptor_log = u;
  return count;
}

// poisson_electrons (include/dvs/photon_noise.cuh:4-9): cuRAND draws in the
// reference's order so seeded streams match a reference build on the same toolkit.
__device__ __forceinline__ double poisson_electrons(curandStateXORWOW_t &rng, double lambda) {
  if (lambda <= 0) return 0;
  if (lambda > 1e6) return fmax(0.0, floor(lambda + sqrt(lambda) * curand_normal_double(&rng) + .5));
  return curand_poisson(&rng, lambda);
}

__global__ void init_pixels_kernel(int n, const int32_t *pixel_of_rank, const double *radiance, PixelParams p,
                                   PhotoParams photo, double stddev, double minimum, unsigned seed, CircuitState st,
                                   int32_t *error) {
  // initialize_pixels (event_sensor.cu:18-28)
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int pixel = pixel_of_rank[k];
  curandStateXORWOW_t rng;
  curand_init(seed, pixel, 0, &rng);
  const double rad = radiance[k];
  if (!isfinite(rad)) {
    atomicOr(error, kErrOptical);
    st.rng[k] = rng;
    return;
  }
  const double u = log(fmax(1e-30, rad * photo.electrons_per_radiance + photo.dark_electrons));
  st.receptor_log[k] = u;
  st.reference_log[k] = u;
  st.refractory_until[k] = -1;
  st.threshold_pos[k] = fmax(minimum, p.threshold_pos + stddev * curand_normal_double(&rng));
  st.threshold_neg[k] = fmax(minimum, p.threshold_neg + stddev * curand_normal_double(&rng));
  st.reset_pending[k] = 0;
  st.rng[k] = rng;
}

__global__ void __launch_bounds__(128) circuit_kernel(int n, const Cell *cells, int c0, int nc,
                                                      const double *radiance, PixelParams p, PhotoParams photo,
                                                      int max_events, CircuitState st, int32_t *ev_count,
                                                      double *slab_t, int8_t *slab_p, int32_t *error,
                                                      unsigned long long *counters) {
  // generate_pixels' circuit half (event_sensor.cu:35-50) over one cell chunk
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int cnt = ev_count[k];
  if (cnt < 0) return;  // failed earlier in this batch
  PixelRegs s{st.receptor_log[k], st.reference_log[k], st.refractory_until[k], st.threshold_pos[k],
              st.threshold_neg[k], st.reset_pending[k] != 0};
  const bool need_rng = photo.shot_noise || p.reset_noise_std > 0;
  curandStateXORWOW_t rng;
  if (need_rng) rng = st.rng[k];
  double *my_t = slab_t + (size_t)k * max_events;
  int8_t *my_p = slab_p + (size_t)k * max_events;
  int failed = 0;
  for (int c = 0; c < nc; ++c) {
    const Cell cell = cells[c0 + c];
    const double rad = radiance[(size_t)c * n + k];
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
  if (need_rng) st.rng[k] = rng;
  if (failed) {
    atomicOr(error, failed);
    ev_count[k] = -1;
  } else {
    ev_count[k] = cnt;
  }
  if (counters && (threadIdx.x & 31) == 0) {
    const int active = min(32, n - (k & ~31));
    atomicAdd(counters + kCntCells, (unsigned long long)active * (unsigned long long)nc);
  }
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

__global__ void __launch_bounds__(128) event_depth_kernel(SceneView S, const dvs_optical_interval *ivs, int n_ivs,
                                                          DevEvent *events, const int32_t *count, int32_t *error,
                                                          unsigned long long *counters) {
  // event-time depth re-trace (event_sensor.cu:51-59); grid-stride over the
  // device-side event count, warps stay converged for the packet traversal.
  float tdist[kStackSlots];
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
    const PixelSample s = sample_pixel_packet<true>(S, pixel, active, pose, tdist);
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

inline int blocks(long long threads, int per_block) { return (int)((threads + per_block - 1) / per_block); }

}  // namespace

// ---- launchers ----------------------------------------------------------------------
cudaError_t launch_pose_from_state(const dvs_optical_state *state, CellPose *out, cudaStream_t s) {
  pose_from_state_kernel<<<1, 32, 0, s>>>(state, out);
  return cudaGetLastError();
}

cudaError_t launch_cell_poses(const dvs_optical_interval *ivs, const Cell *cells, int n, CellPose *out,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  cell_poses_kernel<<<blocks(n, 128), 128, 0, s>>>(ivs, cells, n, out);
  return cudaGetLastError();
}

cudaError_t launch_trace_cells(const SceneView &scene, int n_pix, const CellPose *poses, int c0, int nc, int cw_log2,
                               double *radiance, float *depth, unsigned long long *counters, cudaStream_t s) {
  if (n_pix <= 0 || nc <= 0) return cudaSuccess;
  const int cw = 1 << cw_log2, ppw = 32 >> cw_log2;
  const long long warps = (long long)((n_pix + ppw - 1) / ppw) * ((nc + cw - 1) / cw);
  trace_cells_kernel<<<blocks(warps * 32, 128), 128, 0, s>>>(scene, n_pix, poses, c0, nc, cw_log2, radiance, depth,
                                                              counters);
  return cudaGetLastError();
}

cudaError_t launch_init_pixels(int n, const int32_t *pixel_of_rank, const double *radiance, PixelParams p,
                               PhotoParams photo, double stddev, double minimum, unsigned seed, CircuitState st,
                               int32_t *error, cudaStream_t s) {
  init_pixels_kernel<<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, radiance, p, photo, stddev, minimum, seed, st,
                                                    error);
  return cudaGetLastError();
}

cudaError_t launch_circuit(int n, const Cell *cells, int c0, int nc, const double *radiance, PixelParams p,
                           PhotoParams photo, int max_events, CircuitState st, int32_t *ev_count, double *slab_t,
                           int8_t *slab_p, int32_t *error, unsigned long long *counters, cudaStream_t s) {
  circuit_kernel<<<blocks(n, 128), 128, 0, s>>>(n, cells, c0, nc, radiance, p, photo, max_events, st, ev_count,
                                                slab_t, slab_p, error, counters);
  return cudaGetLastError();
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
  event_depth_kernel<<<sms * 4, 128, 0, s>>>(scene, ivs, n_ivs, events, count, error, counters);
  return cudaGetLastError();
}

cudaError_t launch_radiance_to_float(int n, const int32_t *pixel_of_rank, const double *radiance, const float *depth,
                                     float *image, float *depth_image, cudaStream_t s) {
  radiance_to_float_kernel<<<blocks(n, 128), 128, 0, s>>>(n, pixel_of_rank, radiance, depth, image, depth_image);
  return cudaGetLastError();
}

}  // namespace dvsgb
