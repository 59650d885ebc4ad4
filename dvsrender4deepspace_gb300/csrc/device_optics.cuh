// Device-side optics of the GB300 DVS path: float3 algebra, Hapke, pose
// interpolation, the 8-wide warp-packet BVH traversal and the pixel sample.
// Included by the CUDA translation units that trace rays; everything has
// internal linkage.  Compiled with -fmad=false (see kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

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
// The reference's formulas evaluated through trigonometric identities
// ("identity form"): every transcendental of the phase and azimuth angles
// except acos(cos psi) becomes a square root of a ratio, which the CUDA
// compiler turns into far fewer instructions than tanf/sinf/cosf/powf:
//   tan(acos(c) / 2) = sqrt((1 - c) / (1 + c))      (hapke.hpp:135, :82-84)
//   sin(psi / 2)     = sqrt((1 - cos psi) / 2)       (hapke.hpp:92)
//   cos(psi)         = cos psi (the clamped argument of acos, hapke.hpp:96,123)
//   y^1.5            = y * sqrt(y)                   (hapke.hpp:22-29)
//   e1(y) = exp(-2/pi * q), e2(y) = exp(-1/pi * q^2) with the one quotient
//   q = cot(thetap) cos(y) / sin(y)                  (hapke.hpp:64-73)
// Each is exact in real arithmetic; in FP32 the result stays within a few
// ulp of the reference's own order (bounded against the FP64 oracle in
// tests/test_oracle_golden.py).  The clamps and the one non-finite case keep
// the reference's values: tan(phase/2) is capped at tan(pi/2 - 1e-6)
// (safe_tan, hapke.hpp:14-16), and psi == acos(-1) keeps the reference's
// tan(pi_f / 2) < 0, whose exp overflows and makes the sample NaN (dropped by
// the caller's fmaxf) -- here tan(psi/2) = -inf there.
__device__ __forceinline__ float pow15(float y) { return y * sqrtf(y); }
__device__ __forceinline__ float hg_double_lobe(float cosg, float b, float c) {
  const float one_minus_bb = 1.0f - b * b;
  const float term1 = ((1.0f + c) * 0.5f) * one_minus_bb / pow15(1.0f - 2.0f * b * cosg + b * b);
  const float term2 = ((1.0f - c) * 0.5f) * one_minus_bb / pow15(1.0f + 2.0f * b * cosg + b * b);
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
__device__ __forceinline__ float hfunc(float x, float w, float r0) {
  if (x <= 1e-8f) return 1.0f;
  const float term = r0 + (1.0f - 2.0f * r0 * x) * 0.5f * logf(1.0f + 1.0f / x);
  return 1.0f / (1.0f - w * x * term);
}
__device__ __forceinline__ float hfunc_r0(float w) {
  const float root = sqrtf(fmaxf(0.0f, 1.0f - w));
  return (1.0f - root) / (1.0f + root);
}
__device__ __forceinline__ float porosity_k(float phi) {
  if (phi <= 1e-8f) return 1.0f;
  const float p = 1.209f * powf(phi, 2.0f / 3.0f);
  return -logf(1.0f - p) / p;
}

// The parts of hapke.hpp that depend on the material only: porosity K,
// tan(thetap), 1/tan(thetap), chi(thetap), the r0 of the H-function for the
// scene's single-scattering albedo and the cap of tan(phase/2).  Each is the
// value hapke.hpp recomputes inside every call (same operations, same
// rounding), evaluated once per pixel sample loop instead of per shaded ray.
struct HapkeConst {
  float K, tan_t, cot_t, chi, r0_w, tg_max;
  bool rough;
};
__device__ __forceinline__ HapkeConst hapke_const(const dvs_hapke &p) {
  HapkeConst h;
  h.K = porosity_k(p.phi);
  h.rough = !(p.thetap <= 1e-8f);
  h.tan_t = tanf(p.thetap);
  h.cot_t = 1.0f / h.tan_t;
  h.chi = 1.0f / sqrtf(1.0f + kPi * h.tan_t * h.tan_t);
  h.r0_w = hfunc_r0(p.w);
  h.tg_max = tanf(kPi / 2.0f - 1e-6f);
  return h;
}
// The quotient q = cot(thetap) cos(y) / max(sin(y), 1e-6) shared by e1 and e2.
__device__ __forceinline__ float e_quot(float cot_t, float cosy, float siny) {
  return cot_t * cosy / fmaxf(siny, 1e-6f);
}

// Inlining policy of the large shading and traversal bodies (instruction-cache pressure).
#ifdef DVS_OUTLINE_SHADING
#define DVS_SHADE_INLINE __noinline__
#else
#define DVS_SHADE_INLINE
#endif
// hapke_reflectance (hapke.hpp:131-152) in the identity form above; r0 is
// hfunc's r0 for this albedo.
DVS_SHADE_INLINE __device__ float hapke_reflectance(float cosi, float cose, float cosg, float albedo, float r0,
                                                    const dvs_hapke &p, const HapkeConst &h) {
  if (cosi <= 0 || cose <= 0) return 0;
  cosi = clampf(cosi, 0, 1);
  cose = clampf(cose, 0, 1);
  cosg = clampf(cosg, -1, 1);
  const float sini = sqrtf(fmaxf(0, 1 - cosi * cosi)), sine = sqrtf(fmaxf(0, 1 - cose * cose));
  const float tg = fminf(sqrtf((1.0f - cosg) / (1.0f + cosg)), h.tg_max);
  const float cpsi = clampf((cosg - cosi * cose) / (sini * sine + 1e-6f), -1.0f, 1.0f);
  const float psi = acosf(cpsi);
  const float p_g = hg_double_lobe(cosg, p.b, p.c);
  const float BS = b_s(tg, p.hS);
  // b_c is finite, so with B_C0 == 0 the factor (1 + BC * B_C0) is exactly 1
  // whatever BC is: skip its evaluation.
  const float BC = p.B_C0 != 0.0f ? b_c(tg, p.hC) : 0.0f;
  const float K = h.K;
  float mu0, mue, S;
  if (!h.rough) {
    mu0 = cosi; mue = cose; S = 1.0f;
  } else {
    const float ch = h.chi;
    const float tan_thetap = h.tan_t;
    const float s2 = (1.0f - cpsi) * 0.5f;              // sin^2(psi / 2)
    const float qe = e_quot(h.cot_t, cose, sine), qi = e_quot(h.cot_t, cosi, sini);
    const float e2e = expf((-1.0f / kPi) * qe * qe), e2i = expf((-1.0f / kPi) * qi * qi);
    const float e1e = expf((-2.0f / kPi) * qe), e1i = expf((-2.0f / kPi) * qi);
    // eta(y) = chi * (cos y + sin y * tan(thetap) * e2(y) / (2 - e1(y)))
    const float eta_e = ch * (cose + sine * tan_thetap * e2e / (2.0f - e1e));
    const float eta_i = ch * (cosi + sini * tan_thetap * e2i / (2.0f - e1i));
    const float tpsi = cpsi > -1.0f ? sqrtf((1.0f - cpsi) / (1.0f + cpsi)) : -kInf();  // tan(psi / 2)
    const float fp = expf(-2.0f * tpsi);
    if (cosi >= cose) {
      mu0 = ch * (cosi + sini * tan_thetap * (cpsi * e2e + s2 * e2i) / (2.0f - e1e - (psi / kPi) * e1i));
      mue = ch * (cose + sine * tan_thetap * (e2e - s2 * e2i) / (2.0f - e1e - (psi / kPi) * e1i));
      S = mue / eta_e * cosi / eta_i * ch / (1.0f - fp + fp * ch * (cosi / eta_i));
    } else {
      mu0 = ch * (cosi + sini * tan_thetap * (e2i - s2 * e2e) / (2.0f - e1i - (psi / kPi) * e1e));
      mue = ch * (cose + sine * tan_thetap * (cpsi * e2i + s2 * e2e) / (2.0f - e1i - (psi / kPi) * e1e));
      S = mue / eta_e * cosi / eta_i * ch / (1.0f - fp + fp * ch * (cose / eta_e));
    }
  }
  const float M = hfunc(mu0 / K, albedo, r0) * hfunc(mue / K, albedo, r0) - 1.0f;
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

// Scene geometry formats, as bit flags: the reference's (FP32 child bounds,
// Moller-Trumbore on stored edges), kGeoHalfBounds (FP16 child bounds
// quantised outward against a per-node FP32 origin) and kGeoWatertight (the
// watertight FP32 triangle test on stored vertices), alone or together.
enum GeometryKind : int { kGeoReference = 0, kGeoHalfBounds = 1, kGeoWatertight = 2 };

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

// Watertight ray/triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013) for precision scenes.  The ray
// is sheared onto +z through its origin (kz = the dominant axis of the
// direction, kx/ky swapped when it is negative), the vertices are projected,
// and the signs of the 2-D edge functions U, V, W decide the hit: a ray
// through a shared edge or vertex hits at least one of the triangles.  An edge
// function that rounds to exactly zero is recomputed in FP64 (the products of
// two floats are exact there), as the paper prescribes.  U, V, W weight v0,
// v1, v2, so the reference's barycentrics (u on v1, v on v2) are V/det, W/det.
//
// GB300 layout: a watertight scene stores each triangle three times, its
// vertices in the cyclic axis orders (y,z,x), (z,x,y) and (x,y,z) -- copy kz
// lists axis kz last -- and a ray reads the copy of its dominant axis, so the
// test runs on vertices already in the ray's (kx, ky, kz) order without a
// select per component.  The paper's swap of kx and ky for a negative
// direction only preserves the winding: it negates U, V, W, det and T
// exactly, so t, u and v are the same bits with or without it, and the
// kernels leave it out.
struct WtRay {
  int kz;
  float sx, sy, sz;
};
__device__ __forceinline__ float comp3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
// A vector in the cyclic order whose last axis is kz.
__device__ __forceinline__ float3 wt_perm(float3 v, int kz) {
  return kz == 2 ? v : (kz == 0 ? f3(v.y, v.z, v.x) : f3(v.z, v.x, v.y));
}
__device__ __forceinline__ WtRay wt_setup(float3 d) {
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  WtRay w;
  w.kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  const float3 p = wt_perm(d, w.kz);
  w.sx = p.x / p.z;
  w.sy = p.y / p.z;
  w.sz = 1.0f / p.z;
  return w;
}
// o, v0, v1, v2 in the ray's cyclic order (wt_perm).
__device__ __forceinline__ bool intersect_wt(const WtRay &w, float3 o, float3 v0, float3 v1, float3 v2, float &t,
                                             float &u, float &v) {
  const float3 A = v0 - o, B = v1 - o, C = v2 - o;
  const float az = A.z, bz = B.z, cz = C.z;
  const float ax = A.x - w.sx * az, ay = A.y - w.sy * az;
  const float bx = B.x - w.sx * bz, by = B.y - w.sy * bz;
  const float cx = C.x - w.sx * cz, cy = C.y - w.sy * cz;
  float U = cx * by - cy * bx, V = ax * cy - ay * cx;
  // A nonzero float edge function has the sign of the exact one (rounding
  // keeps the order of the two products), and so does its FP64 recomputation:
  // opposite nonzero signs of U and V are a miss whatever W is, decided
  // before W is formed.
  if ((U < 0.0f && V > 0.0f) || (U > 0.0f && V < 0.0f)) return false;
  float W = bx * ay - by * ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)cx * (double)by - (double)cy * (double)bx);
    V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
    W = (float)((double)bx * (double)ay - (double)by * (double)ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = U + V + W;
  if (det == 0.0f) return false;
  const float T = U * (w.sz * az) + V * (w.sz * bz) + W * (w.sz * cz);
  const float rcp = 1.0f / det;
  t = T * rcp;
  if (!(t > kRayEps)) return false;
  u = V * rcp;
  v = W * rcp;
  return true;
}
// One leaf-order triangle record against one ray.  Records hold (v0, e1, e2),
// or in watertight scenes (v0, v1, v2) in the ray's cyclic order; o is the
// ray origin, op the origin in that order (watertight scenes).
template <int kGeo>
__device__ __forceinline__ bool tri_hit(const WtRay &w, float3 d, float3 o, float3 op, float4 a, float4 b, float4 q,
                                        float &t, float &u, float &v) {
  if constexpr (!(kGeo & kGeoWatertight))
    return intersect_tri(d, o, f3(a.x, a.y, a.z), f3(a.w, b.x, b.y), f3(b.z, b.w, q.x), t, u, v);
  else
    return intersect_wt(w, op, f3(a.x, a.y, a.z), f3(a.w, b.x, b.y), f3(b.z, b.w, q.x), t, u, v);
}
template <int kGeo>
__device__ __forceinline__ WtRay wt_ray(float3 d) {
  if constexpr (!(kGeo & kGeoWatertight)) return WtRay{2, 0.f, 0.f, 0.f};
  else return wt_setup(d);
}
template <int kGeo>
__device__ __forceinline__ float3 wt_origin(const WtRay &w, float3 o) {
  if constexpr (!(kGeo & kGeoWatertight)) return o;
  else return wt_perm(o, w.kz);
}
// The record of leaf-order triangle `tri` a ray with dominant axis kz reads:
// the single record, or in watertight scenes its copy kz (copy 2 holds the
// vertices in world order).
template <int kGeo>
__device__ __forceinline__ const float4 *tri_record(const SceneView &S, int tri, int kz) {
  if constexpr (!(kGeo & kGeoWatertight)) return reinterpret_cast<const float4 *>(S.tris + tri);
  else return reinterpret_cast<const float4 *>(S.tris + 3 * (size_t)tri + kz);
}

// ---- 8-wide packet traversal ------------------------------------------------------
// Float min/max across a warp through order-preserving unsigned keys.
__device__ __forceinline__ unsigned ford(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float funord(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ float wmin(float x) { return funord(__reduce_min_sync(kFull, ford(x))); }
__device__ __forceinline__ float wmax(float x) { return funord(__reduce_max_sync(kFull, ford(x))); }

struct ChildRec {
  float3 lo, hi;
  int child, count;
};
__device__ __forceinline__ float half_bits_to_float(unsigned bits) {
  return __half2float(__ushort_as_half((unsigned short)(bits & 0xffffu)));
}
// Child record `slot` of node `node`.  Precision nodes decode each bound as
// origin + offset with the addition rounded toward -inf (lower bounds) or +inf
// (upper bounds); the builder rounded the offsets the same way, so a decoded
// box always contains the exact FP32 box and no ray misses a child it would
// enter (the leaf's triangles are then tested in FP32).
template <int kGeo>
__device__ __forceinline__ ChildRec load_child(const SceneView &S, int node, int slot) {
  ChildRec r;
  if constexpr (!(kGeo & kGeoHalfBounds)) {
    const float4 *p = reinterpret_cast<const float4 *>(&S.nodes[node].c[slot]);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    r.lo = f3(a.x, a.y, a.z);
    r.hi = f3(a.w, b.x, b.y);
    r.child = __float_as_int(b.z);
    r.count = __float_as_int(b.w);
  } else {
    const float4 org = __ldg(reinterpret_cast<const float4 *>(S.qnodes + node));
    const uint4 c = __ldg(reinterpret_cast<const uint4 *>(&S.qnodes[node].c[slot]));
    r.lo = f3(__fadd_rd(org.x, half_bits_to_float(c.x)), __fadd_rd(org.y, half_bits_to_float(c.x >> 16)),
              __fadd_rd(org.z, half_bits_to_float(c.y)));
    r.hi = f3(__fadd_ru(org.x, half_bits_to_float(c.y >> 16)), __fadd_ru(org.y, half_bits_to_float(c.z)),
              __fadd_ru(org.z, half_bits_to_float(c.z >> 16)));
    const unsigned link = c.w;
    if (link == kQLinkEmpty) {
      r.child = 0;
      r.count = -1;
    } else if (link & kQLinkLeaf) {
      r.child = (int)(link & kQLinkFirstMask);
      r.count = (int)((link >> kQLinkCountShift) & 15u) + 1;
    } else {
      r.child = (int)link;
      r.count = 0;
    }
  }
  return r;
}

// Slab test of one ray (device_ray.hpp:21-29 form).
__device__ __forceinline__ bool slab(float3 lo, float3 hi, float3 o, float3 idir, float t_min, float t_max,
                                     float &tnear) {
  float tx0 = (lo.x - o.x) * idir.x, tx1 = (hi.x - o.x) * idir.x;
  float ty0 = (lo.y - o.y) * idir.y, ty1 = (hi.y - o.y) * idir.y;
  float tz0 = (lo.z - o.z) * idir.z, tz1 = (hi.z - o.z) * idir.z;
  float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  tmin = fmaxf(t_min, tmin);
  tmax = fminf(t_max, tmax);
  tnear = tmin;
  return tmax >= tmin;
}

// The rays of a warp as intervals of origin and inverse direction.  A child
// is entered when some ray of the box could hit it: every bound is an
// extreme of the same rounded operations each ray performs, so the packet
// never culls a node that one of its rays would enter.
//
// Packets use interval tests only when each axis' inverse direction keeps
// one sign across the packet.  Where a direction component changes sign
// inside the packet (near-axial rays, e.g. the image centre of a nadir
// camera) its inverse spans -1e20..1e20 and that axis culls nothing, so such
// packets take the per-ray path.
struct Packet {
  float3 olo, ohi, ilo, ihi;
  // per axis: the origin bound that gives the earliest entry (o_near) and
  // the latest exit (o_far), and whether the direction is negative
  float3 o_near, o_far;
  bool nx, ny, nz;
  bool coherent;
};
// Interval slab bounds of one axis for a packet whose inverse direction has
// one sign: the entry plane is the near one for every ray, and the extreme
// of the four corner products (lo/hi plane offset x ilo/ihi) is the one
// picked by the sign of the plane offset.  Rounded subtraction and
// multiplication are monotone, so L and U equal the four-product interval
// bounds (up to the sign of a zero) with a third of the arithmetic.
__device__ __forceinline__ void axis_bounds_fixed(float lo, float hi, bool neg, float on, float of, float ilo,
                                                  float ihi, float &L, float &U) {
  const float aN = (neg ? hi : lo) - on;
  const float aF = (neg ? lo : hi) - of;
  L = aN * (aN >= 0.0f ? ilo : ihi);
  U = aF * (aF >= 0.0f ? ihi : ilo);
}
__device__ __forceinline__ bool packet_slab(const ChildRec &c, const Packet &P, float t_min, float t_max,
                                            float &tnear) {
  float Lx, Ux, Ly, Uy, Lz, Uz;
  axis_bounds_fixed(c.lo.x, c.hi.x, P.nx, P.o_near.x, P.o_far.x, P.ilo.x, P.ihi.x, Lx, Ux);
  axis_bounds_fixed(c.lo.y, c.hi.y, P.ny, P.o_near.y, P.o_far.y, P.ilo.y, P.ihi.y, Ly, Uy);
  axis_bounds_fixed(c.lo.z, c.hi.z, P.nz, P.o_near.z, P.o_far.z, P.ilo.z, P.ihi.z, Lz, Uz);
  const float lb = fmaxf(fmaxf(fmaxf(Lx, Ly), Lz), t_min);
  const float ub = fminf(fminf(fminf(Ux, Uy), Uz), t_max);
  tnear = lb;
  return ub >= lb;
}
// Warp minimum and maximum of one value from one order-preserving key;
// inactive lanes count as +inf for the minimum and -inf for the maximum.
__device__ __forceinline__ void wminmax(float x, bool active, float &lo, float &hi) {
  const unsigned k = ford(x);
  lo = funord(__reduce_min_sync(kFull, active ? k : 0xff800000u));  // ford(+inf)
  hi = funord(__reduce_max_sync(kFull, active ? k : 0x007fffffu));  // ford(-inf)
}
__device__ Packet make_packet(const SceneView &S, float3 o, float3 d, float3 idir, bool active) {
  Packet P;
  wminmax(o.x, active, P.olo.x, P.ohi.x);
  wminmax(o.y, active, P.olo.y, P.ohi.y);
  wminmax(o.z, active, P.olo.z, P.ohi.z);
  wminmax(idir.x, active, P.ilo.x, P.ihi.x);
  wminmax(idir.y, active, P.ilo.y, P.ihi.y);
  wminmax(idir.z, active, P.ilo.z, P.ihi.z);
  float dlo, dhi;
  wminmax(d.x, active, dlo, dhi);
  const float dx = dhi - dlo;
  wminmax(d.y, active, dlo, dhi);
  const float dy = dhi - dlo;
  wminmax(d.z, active, dlo, dhi);
  const float dz = dhi - dlo;
  const float ds = fmaxf(fmaxf(dx, dy), dz);
  const float os = fmaxf(fmaxf(P.ohi.x - P.olo.x, P.ohi.y - P.olo.y), P.ohi.z - P.olo.z);
  P.nx = P.ihi.x < 0.0f;
  P.ny = P.ihi.y < 0.0f;
  P.nz = P.ihi.z < 0.0f;
  const bool one_sign = (P.nx || P.ilo.x > 0.0f) && (P.ny || P.ilo.y > 0.0f) && (P.nz || P.ilo.z > 0.0f);
  // bundles whose footprint stays within a small fraction of the scene
  P.coherent = one_sign && ds <= 0.02f && os <= S.coherent_span;
  P.o_near = f3(P.nx ? P.olo.x : P.ohi.x, P.ny ? P.olo.y : P.ohi.y, P.nz ? P.olo.z : P.ohi.z);
  P.o_far = f3(P.nx ? P.ohi.x : P.olo.x, P.ny ? P.ohi.y : P.olo.y, P.nz ? P.ohi.z : P.olo.z);
  return P;
}

// Warp-uniform traversal stack in shared memory: node codes and the packet's
// entry distance.  Inner node: index >= 0; leaf: -(node * 8 + slot) - 1.
struct Stack {
  int *code;
  float *t;
  int sp;
};
__device__ __forceinline__ int leaf_code(int node, int slot) { return -(node * kBvhWidth + slot) - 1; }

struct HitRecord {
  int hit;  // 1 hit, 0 miss, -1 stack overflow (device_ray.hpp:152)
  int tri;
  float t, u, v;
};

// Expands an inner node: children the packet may hit are ordered near to far;
// all but the nearest go on the stack.  Returns false when none is hit.
// Coherent packets test one child per lane (lanes 0..7) with interval bounds;
// others test every child per ray and take the warp minimum as the key.
template <bool kSorted, int kGeo>
__device__ __forceinline__ bool expand_node(const SceneView &S, int node, const Packet &P, float3 o, float3 idir,
                                            bool lane_live, float t_min, float lane_tmax, float packet_tmax,
                                            Stack &st, int &next, float &next_t, bool &overflow) {
  const int lane = threadIdx.x & 31;
  float key = kInf();
  bool hit = false;
  int code = 0;
  if (P.coherent) {
    if (lane < kBvhWidth) {
      const ChildRec c = load_child<kGeo>(S, node, lane);
      if (c.count >= 0) {
        hit = packet_slab(c, P, t_min, packet_tmax, key);
        code = c.count > 0 ? leaf_code(node, lane) : c.child;
      }
    }
  } else {
    for (int slot = 0; slot < kBvhWidth; ++slot) {
      const ChildRec c = load_child<kGeo>(S, node, slot);
      float tn = kInf();
      const bool h = c.count >= 0 && lane_live && slab(c.lo, c.hi, o, idir, t_min, lane_tmax, tn);
      const float k = wmin(h ? tn : kInf());
      if (lane == slot) {
        hit = k < kInf();
        key = k;
        code = c.count > 0 ? leaf_code(node, slot) : c.child;
      }
    }
  }
  const unsigned mask = __ballot_sync(kFull, hit && lane < kBvhWidth);
  if (!mask) return false;
  const int n = __popc(mask);
  if (n == 1) {  // the common case of a thin packet: nothing to order or push
    const int only = __ffs(mask) - 1;
    next = __shfl_sync(kFull, code, only);
    next_t = __shfl_sync(kFull, key, only);
    return true;
  }
  int rank = 0;
  if (kSorted) {
#pragma unroll
    for (int j = 0; j < kBvhWidth; ++j) {
      const float kj = __shfl_sync(kFull, key, j);
      rank += ((mask >> j) & 1) && (kj < key || (kj == key && j < lane)) ? 1 : 0;
    }
  } else {
    rank = __popc(mask & ((1u << lane) - 1u));
  }
  if (st.sp + n - 1 > kStackSlots) {
    overflow = true;
    return false;
  }
  if (hit && lane < kBvhWidth && rank > 0) {
    const int slot = st.sp + (n - 1 - rank);
    st.code[slot] = code;
    st.t[slot] = key;
  }
  const int first = __ffs(__ballot_sync(kFull, hit && lane < kBvhWidth && rank == 0)) - 1;
  next = __shfl_sync(kFull, code, first);
  next_t = __shfl_sync(kFull, key, first);
  st.sp += n - 1;
  __syncwarp();
  return true;
}

// Nearest hit for the rays of a warp (trace_nearest, device_ray.hpp:136-158).
// All 32 lanes call converged; inactive lanes never hit.  Each lane tests a
// leaf's triangles only when its own slab test reaches the leaf.
template <int kGeo>
__device__ HitRecord trace_nearest_packet(const SceneView &S, float3 o, float3 d, bool active, int *stack_code,
                                          float *stack_t) {
  const float3 idir = inverse_direction(d);
  const WtRay wr = wt_ray<kGeo>(d);
  const float3 op = wt_origin<kGeo>(wr, o);
  float closest = active ? 1e30f : -1.0f;
  HitRecord h{0, -1, 0.f, 0.f, 0.f};
  const Packet P = make_packet(S, o, d, idir, active);
  float packet_tmax = wmax(active ? closest : -1.0f);
  Stack st{stack_code, stack_t, 0};
  int entry = 0;
  float entry_t = 0.0f;
  bool overflow = false;
  while (true) {
    if (entry_t <= packet_tmax) {
      if (entry >= 0) {
        int next;
        float next_t;
        if (expand_node<true, kGeo>(S, entry, P, o, idir, active, kRayEps, closest, packet_tmax, st, next, next_t,
                              overflow)) {
          entry = next;
          entry_t = next_t;
          continue;
        }
        if (overflow) break;
      } else {
        const int lc = -entry - 1;
        const ChildRec c = load_child<kGeo>(S, lc / kBvhWidth, lc % kBvhWidth);
        float tn;
        const bool need = active && slab(c.lo, c.hi, o, idir, kRayEps, closest, tn);
        for (int i = 0; i < c.count; ++i) {
          const float4 *r = tri_record<kGeo>(S, c.child + i, wr.kz);
          const float4 a = __ldg(r), b = __ldg(r + 1), q = __ldg(r + 2);
          float t, u, v;
          if (need && tri_hit<kGeo>(wr, d, o, op, a, b, q, t, u, v) && t < closest) {
            closest = t;
            h.hit = 1; h.tri = c.child + i; h.t = t; h.u = u; h.v = v;
          }
        }
        packet_tmax = wmax(active ? closest : -1.0f);
      }
    }
    if (st.sp == 0) break;
    --st.sp;
    entry = st.code[st.sp];
    entry_t = st.t[st.sp];
  }
  __syncwarp();
  if (overflow) h.hit = -1;
  return h;
}

// Any hit toward the light (trace_shadow_ray_any_hit, device_ray.hpp:81-135):
// skips the camera-hit triangle, t in (kRayEps, 1e30); overflow counts as occluded.
template <int kGeo>
DVS_SHADE_INLINE __device__ bool trace_shadow_packet(const SceneView &S, float3 o, float3 d, bool active, int self,
                                                     int *stack_code, float *stack_t) {
  const float3 idir = inverse_direction(d);
  const WtRay wr = wt_ray<kGeo>(d);
  const float3 op = wt_origin<kGeo>(wr, o);
  bool alive = active;
  bool occluded = false;
  const float t_max = 1e30f;
  const Packet P = make_packet(S, o, d, idir, active);
  Stack st{stack_code, stack_t, 0};
  int entry = 0;
  float entry_t = 0.0f;
  bool overflow = false;
  while (__any_sync(kFull, alive)) {
    if (entry >= 0) {
      int next;
      float next_t;
      if (expand_node<false, kGeo>(S, entry, P, o, idir, alive, kRayEps, alive ? t_max : -1.0f, t_max, st, next, next_t,
                             overflow)) {
        entry = next;
        entry_t = next_t;
        continue;
      }
      if (overflow) {
        occluded = occluded || alive;  // conservative (device_ray.hpp:119)
        break;
      }
    } else {
      const int lc = -entry - 1;
      const ChildRec c = load_child<kGeo>(S, lc / kBvhWidth, lc % kBvhWidth);
      float tn;
      const bool need = alive && slab(c.lo, c.hi, o, idir, kRayEps, t_max, tn);
      for (int i = 0; i < c.count; ++i) {
        const int id = c.child + i;
        const float4 *r = tri_record<kGeo>(S, id, wr.kz);
        const float4 a = __ldg(r), b = __ldg(r + 1), q = __ldg(r + 2);
        float t, u, v;
        if (need && alive && id != self &&
            tri_hit<kGeo>(wr, d, o, op, a, b, q, t, u, v) && t > kRayEps &&
            t < t_max) {
          occluded = true;
          alive = false;
        }
      }
    }
    if (st.sp == 0) break;
    --st.sp;
    entry = st.code[st.sp];
    entry_t = st.t[st.sp];
  }
  (void)entry_t;
  __syncwarp();
  return occluded;
}


// shadow_origin (device_optics.cuh:37-51) from the leaf-order triangle record.
__device__ float3 shadow_origin(float3 a, float3 e1, float3 e2, float u, float v, float3 light) {
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

// shadow_origin from a record (a, b, c = its three float4s): the edges are
// stored, or v1 - v0, v2 - v0 with the same float subtraction (watertight
// scenes), so both give the reference's edge bits.
template <int kGeo>
__device__ __forceinline__ float3 shadow_origin_rec(float4 a, float4 b, float4 c, float u, float v, float3 light) {
  const float3 v0 = f3(a.x, a.y, a.z), p = f3(a.w, b.x, b.y), q = f3(b.z, b.w, c.x);
  if constexpr (!(kGeo & kGeoWatertight)) return shadow_origin(v0, p, q, u, v, light);
  else return shadow_origin(v0, p - v0, q - v0, u, v, light);
}

struct PixelSample {
  double radiance;
  float depth;
  bool valid;
  unsigned primary, shadow;
};

// What one pixel sample produces.
enum SampleMode : int { kRadiance = 0, kRadianceDepth = 1, kDepthOnly = 2 };

// cos^4 field falloff (device_optics.cuh:90) in FP64, as the reference.
__device__ __forceinline__ double cos4_of(float px, float py) {
  return 1.0 / ((1.0 + px * px + py * py) * (1.0 + px * px + py * py));
}
// One sub-ray of a pixel: its image-plane coordinates and FP64 cos^4, the
// same values subray_x/subray_y/cos4_of give.  A warp whose lanes all sample
// one pixel forms them once per sub-ray in shared memory instead of once per
// lane and ray (an integer division by the sub-ray count and four IEEE
// divisions per ray).
struct SubraySample {
  double cos4;
  float px, py;
};
__device__ __forceinline__ float subray_x(const SceneView &S, int px_i, int sx) {
  return (px_i + (sx + .5f) / S.samples - .5f - S.cx) / S.fx;
}
__device__ __forceinline__ float subray_y(const SceneView &S, int py_i, int sy) {
  return (py_i + (sy + .5f) / S.samples - .5f - S.cy) / S.fy;
}

// sample_pixel (device_optics.cuh:73-94) for one lane of a converged warp.
// subrays: when every lane of the warp samples the same pixel, its sub-rays'
// coordinates and cos^4, formed once per warp (shared memory); otherwise nullptr.
template <int kMode, int kGeo = kGeoReference>
__device__ PixelSample sample_pixel_packet(const SceneView &S, int pixel, bool active, const CellPose &pose,
                                           int *stack_code, float *stack_t, const SubraySample *subrays) {
  PixelSample out{0.0, -1.0f, true, 0u, 0u};
  double depth = 0;
  int valid_depth = 0;
  const float3 light = f3(pose.lx, pose.ly, pose.lz);
  const float3 origin = f3(pose.px, pose.py, pose.pz);
  const int ss = S.samples;
  const int px_i = pixel % S.width, py_i = pixel / S.width;
  const HapkeConst hc = hapke_const(S.hapke);
  const float3 lnorm = normalize(light);  // as in sample_pixel_group
  for (int sy = 0; sy < ss; ++sy)
    for (int sx = 0; sx < ss; ++sx) {
      const float px = subrays ? subrays[sy * ss + sx].px : subray_x(S, px_i, sx);
      const float py = subrays ? subrays[sy * ss + sx].py : subray_y(S, py_i, sy);
      const float3 ray = normalize(rotate_ray(pose, f3(px, -py, -1)));
      const HitRecord hit = trace_nearest_packet<kGeo>(S, origin, ray, active && out.valid, stack_code, stack_t);
      if (active && out.valid) ++out.primary;
      if (hit.hit < 0) out.valid = false;
      const bool hitp = active && out.valid && hit.hit == 1;
      bool lit = false;
      float3 normal = f3(0, 0, 0), sorigin = f3(0, 0, 0);
      float albedo = S.hapke.w, r0 = hc.r0_w;
      if (hitp) {
        if (kMode != kRadiance) {
          depth += hit.t;
          ++valid_depth;
        }
        if (kMode != kDepthOnly) {
          const ShadeRecord *sr = S.shade + hit.tri;
          const float4 *q = reinterpret_cast<const float4 *>(sr);
          const float4 s0 = __ldg(q), s1 = __ldg(q + 1), s2 = __ldg(q + 2);
          const float w = 1 - hit.u - hit.v;
          normal = normalize(f3(s0.x, s0.y, s0.z) * w + f3(s1.x, s1.y, s1.z) * hit.u + f3(s2.x, s2.y, s2.z) * hit.v);
          lit = !(dot(normal, light) <= 0 || dot(normal, -ray) <= 0);
          if (lit) {
            const float4 *r = tri_record<kGeo>(S, hit.tri, 2);
            const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
            sorigin = shadow_origin_rec<kGeo>(a, b, c, hit.u, hit.v, light);
            if (S.has_albedo) {
              albedo = s0.w * w + s1.w * hit.u + s2.w * hit.v;
              r0 = hfunc_r0(albedo);
            }
          }
        }
      }
      if (kMode != kDepthOnly) {
        if (__any_sync(kFull, lit)) {
          if (lit) ++out.shadow;
          const bool occ = trace_shadow_packet<kGeo>(S, sorigin, light, lit, hit.tri, stack_code, stack_t);
          if (lit && !occ) {
            const double cos4 = subrays ? subrays[sy * ss + sx].cos4 : cos4_of(px, py);
            // hapke_directional_reflectance (hapke.hpp:153-157)
            const float3 n = normalize(normal), l = lnorm, v = normalize(-ray);
            const float n_h = hapke_reflectance(dot(n, l), dot(n, v), dot(l, v), albedo, r0, S.hapke, hc);
            out.radiance += fmaxf(0, n_h * pose.intensity) * cos4;
          }
        }
      }
    }
  out.radiance /= ss * ss;
  out.depth = valid_depth ? float(depth / valid_depth) : -1.0f;
  return out;
}

// ---- two sub-rays per lane ------------------------------------------------------
// The same traversal with each lane carrying R rays (two neighbouring sub-rays
// of its pixel-cell): the packet is 32 x R rays, so the interval node tests,
// the stack traffic and the packet set-up are paid once per 32 x R rays, and
// a leaf's triangle records are loaded once for the lane's R rays.  Per-ray
// results are those of the one-ray traversal (every interval bound covers
// all R rays; leaves are tested per ray).

// Warp extremes of per-lane [lo, hi] ranges; inactive lanes count as empty.
__device__ __forceinline__ void wrange(float lo, float hi, bool active, float &wlo, float &whi) {
  wlo = funord(__reduce_min_sync(kFull, active ? ford(lo) : 0xff800000u));
  whi = funord(__reduce_max_sync(kFull, active ? ford(hi) : 0x007fffffu));
}

template <int R>
__device__ Packet make_packet_r(const SceneView &S, const float3 (&o)[R], const float3 (&d)[R],
                                const float3 (&idir)[R], const bool (&active)[R]) {
  float3 olo = f3(kInf(), kInf(), kInf()), ohi = -olo, ilo = olo, ihi = -olo, dlo = olo, dhi = -olo;
  bool any = false;
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (active[r]) {
      any = true;
      olo = f3(fminf(olo.x, o[r].x), fminf(olo.y, o[r].y), fminf(olo.z, o[r].z));
      ohi = f3(fmaxf(ohi.x, o[r].x), fmaxf(ohi.y, o[r].y), fmaxf(ohi.z, o[r].z));
      ilo = f3(fminf(ilo.x, idir[r].x), fminf(ilo.y, idir[r].y), fminf(ilo.z, idir[r].z));
      ihi = f3(fmaxf(ihi.x, idir[r].x), fmaxf(ihi.y, idir[r].y), fmaxf(ihi.z, idir[r].z));
      dlo = f3(fminf(dlo.x, d[r].x), fminf(dlo.y, d[r].y), fminf(dlo.z, d[r].z));
      dhi = f3(fmaxf(dhi.x, d[r].x), fmaxf(dhi.y, d[r].y), fmaxf(dhi.z, d[r].z));
    }
  Packet P;
  wrange(olo.x, ohi.x, any, P.olo.x, P.ohi.x);
  wrange(olo.y, ohi.y, any, P.olo.y, P.ohi.y);
  wrange(olo.z, ohi.z, any, P.olo.z, P.ohi.z);
  wrange(ilo.x, ihi.x, any, P.ilo.x, P.ihi.x);
  wrange(ilo.y, ihi.y, any, P.ilo.y, P.ihi.y);
  wrange(ilo.z, ihi.z, any, P.ilo.z, P.ihi.z);
  float wl, wh;
  wrange(dlo.x, dhi.x, any, wl, wh);
  const float dx = wh - wl;
  wrange(dlo.y, dhi.y, any, wl, wh);
  const float dy = wh - wl;
  wrange(dlo.z, dhi.z, any, wl, wh);
  const float dz = wh - wl;
  const float ds = fmaxf(fmaxf(dx, dy), dz);
  const float os = fmaxf(fmaxf(P.ohi.x - P.olo.x, P.ohi.y - P.olo.y), P.ohi.z - P.olo.z);
  P.nx = P.ihi.x < 0.0f;
  P.ny = P.ihi.y < 0.0f;
  P.nz = P.ihi.z < 0.0f;
  const bool one_sign = (P.nx || P.ilo.x > 0.0f) && (P.ny || P.ilo.y > 0.0f) && (P.nz || P.ilo.z > 0.0f);
  P.coherent = one_sign && ds <= 0.02f && os <= S.coherent_span;
  P.o_near = f3(P.nx ? P.olo.x : P.ohi.x, P.ny ? P.olo.y : P.ohi.y, P.nz ? P.olo.z : P.ohi.z);
  P.o_far = f3(P.nx ? P.ohi.x : P.olo.x, P.ny ? P.ohi.y : P.olo.y, P.nz ? P.ohi.z : P.olo.z);
  return P;
}

template <bool kSorted, int R, int kGeo>
__device__ __forceinline__ bool expand_node_r(const SceneView &S, int node, const Packet &P, const float3 (&o)[R],
                                              const float3 (&idir)[R], const bool (&live)[R], float t_min,
                                              const float (&lane_tmax)[R], float packet_tmax, Stack &st, int &next,
                                              float &next_t, bool &overflow) {
  const int lane = threadIdx.x & 31;
  float key = kInf();
  bool hit = false;
  int code = 0;
  if (P.coherent) {
    if (lane < kBvhWidth) {
      const ChildRec c = load_child<kGeo>(S, node, lane);
      if (c.count >= 0) {
        hit = packet_slab(c, P, t_min, packet_tmax, key);
        code = c.count > 0 ? leaf_code(node, lane) : c.child;
      }
    }
  } else {
    for (int slot = 0; slot < kBvhWidth; ++slot) {
      const ChildRec c = load_child<kGeo>(S, node, slot);
      float near = kInf();
#pragma unroll
      for (int r = 0; r < R; ++r) {
        float tn = kInf();
        if (c.count >= 0 && live[r] && slab(c.lo, c.hi, o[r], idir[r], t_min, lane_tmax[r], tn)) near = fminf(near, tn);
      }
      const float k = wmin(near);
      if (lane == slot) {
        hit = k < kInf();
        key = k;
        code = c.count > 0 ? leaf_code(node, slot) : c.child;
      }
    }
  }
  const unsigned mask = __ballot_sync(kFull, hit && lane < kBvhWidth);
  if (!mask) return false;
  const int n = __popc(mask);
  if (n == 1) {
    const int only = __ffs(mask) - 1;
    next = __shfl_sync(kFull, code, only);
    next_t = __shfl_sync(kFull, key, only);
    return true;
  }
  int rank = 0;
  if (kSorted) {
#pragma unroll
    for (int j = 0; j < kBvhWidth; ++j) {
      const float kj = __shfl_sync(kFull, key, j);
      rank += ((mask >> j) & 1) && (kj < key || (kj == key && j < lane)) ? 1 : 0;
    }
  } else {
    rank = __popc(mask & ((1u << lane) - 1u));
  }
  if (st.sp + n - 1 > kStackSlots) {
    overflow = true;
    return false;
  }
  if (hit && lane < kBvhWidth && rank > 0) {
    const int slot = st.sp + (n - 1 - rank);
    st.code[slot] = code;
    st.t[slot] = key;
  }
  const int first = __ffs(__ballot_sync(kFull, hit && lane < kBvhWidth && rank == 0)) - 1;
  next = __shfl_sync(kFull, code, first);
  next_t = __shfl_sync(kFull, key, first);
  st.sp += n - 1;
  __syncwarp();
  return true;
}

template <int R>
__device__ __forceinline__ float lane_reach(const bool (&active)[R], const float (&closest)[R]) {
  float m = -1.0f;
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (active[r]) m = fmaxf(m, closest[r]);
  return m;
}

template <int R, int kGeo>
__device__ void trace_nearest_packet_r(const SceneView &S, const float3 (&o)[R], const float3 (&d)[R],
                                       const bool (&active)[R], int *stack_code, float *stack_t, HitRecord (&h)[R]) {
  float3 idir[R], op[R];
  float closest[R];
  WtRay wr[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    idir[r] = inverse_direction(d[r]);
    wr[r] = wt_ray<kGeo>(d[r]);
    op[r] = wt_origin<kGeo>(wr[r], o[r]);
    closest[r] = active[r] ? 1e30f : -1.0f;
    h[r] = HitRecord{0, -1, 0.f, 0.f, 0.f};
  }
  const Packet P = make_packet_r<R>(S, o, d, idir, active);
  float packet_tmax = wmax(lane_reach<R>(active, closest));
  Stack st{stack_code, stack_t, 0};
  int entry = 0;
  float entry_t = 0.0f;
  bool overflow = false;
  while (true) {
    if (entry_t <= packet_tmax) {
      if (entry >= 0) {
        int next;
        float next_t;
        if (expand_node_r<true, R, kGeo>(S, entry, P, o, idir, active, kRayEps, closest, packet_tmax, st, next, next_t,
                                   overflow)) {
          entry = next;
          entry_t = next_t;
          continue;
        }
        if (overflow) break;
      } else {
        const int lc = -entry - 1;
        const ChildRec c = load_child<kGeo>(S, lc / kBvhWidth, lc % kBvhWidth);
        bool need[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          float tn;
          need[r] = active[r] && slab(c.lo, c.hi, o[r], idir[r], kRayEps, closest[r], tn);
        }
        for (int i = 0; i < c.count; ++i) {
          // one record per lane for all its rays; a ray of another dominant
          // axis (watertight scenes, rare inside a lane) reads its own copy
          const float4 *q4 = tri_record<kGeo>(S, c.child + i, wr[0].kz);
          float4 a = __ldg(q4), b = __ldg(q4 + 1), q = __ldg(q4 + 2);
          int loaded = wr[0].kz;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if constexpr ((kGeo & kGeoWatertight) != 0) {
              if (wr[r].kz != loaded) {
                const float4 *p4 = tri_record<kGeo>(S, c.child + i, wr[r].kz);
                a = __ldg(p4);
                b = __ldg(p4 + 1);
                q = __ldg(p4 + 2);
                loaded = wr[r].kz;
              }
            }
            float t, u, v;
            if (need[r] && tri_hit<kGeo>(wr[r], d[r], o[r], op[r], a, b, q, t, u, v) && t < closest[r]) {
              closest[r] = t;
              h[r].hit = 1; h[r].tri = c.child + i; h[r].t = t; h[r].u = u; h[r].v = v;
            }
          }
        }
        packet_tmax = wmax(lane_reach<R>(active, closest));
      }
    }
    if (st.sp == 0) break;
    --st.sp;
    entry = st.code[st.sp];
    entry_t = st.t[st.sp];
  }
  __syncwarp();
  if (overflow)
#pragma unroll
    for (int r = 0; r < R; ++r) h[r].hit = -1;
}

// The direction terms of a lane's shadow rays (all toward the same light):
// formed once per pixel sample loop, not once per shadow packet.
struct ShadowDir {
  float3 idir;
  WtRay wr;
};
template <int kGeo>
__device__ __forceinline__ ShadowDir shadow_dir(float3 light) {
  return ShadowDir{inverse_direction(light), wt_ray<kGeo>(light)};
}

template <int R, int kGeo>
__device__ void trace_shadow_packet_r(const SceneView &S, const float3 (&o)[R], float3 light, const ShadowDir &sd,
                                      const bool (&active)[R], const int (&self)[R], int *stack_code, float *stack_t,
                                      bool (&occluded)[R]) {
  const float3 idir1 = sd.idir;
  const WtRay wr = sd.wr;
  float3 d[R], idir[R], op[R];
  bool alive[R];
  float reach[R];
  const float t_max = 1e30f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    d[r] = light;
    idir[r] = idir1;
    op[r] = wt_origin<kGeo>(wr, o[r]);
    alive[r] = active[r];
    occluded[r] = false;
  }
  const Packet P = make_packet_r<R>(S, o, d, idir, active);
  Stack st{stack_code, stack_t, 0};
  int entry = 0;
  bool overflow = false;
  while (true) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; ++r) any = any || alive[r];
    if (!__any_sync(kFull, any)) break;
    if (entry >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) reach[r] = alive[r] ? t_max : -1.0f;
      int next;
      float next_t;
      if (expand_node_r<false, R, kGeo>(S, entry, P, o, idir, alive, kRayEps, reach, t_max, st, next, next_t, overflow)) {
        entry = next;
        continue;
      }
      if (overflow) {
#pragma unroll
        for (int r = 0; r < R; ++r) occluded[r] = occluded[r] || alive[r];  // conservative (device_ray.hpp:119)
        break;
      }
    } else {
      const int lc = -entry - 1;
      const ChildRec c = load_child<kGeo>(S, lc / kBvhWidth, lc % kBvhWidth);
      bool need[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        float tn;
        need[r] = alive[r] && slab(c.lo, c.hi, o[r], idir[r], kRayEps, t_max, tn);
      }
      for (int i = 0; i < c.count; ++i) {
        const int id = c.child + i;
        const float4 *q4 = tri_record<kGeo>(S, id, wr.kz);
        const float4 a = __ldg(q4), b = __ldg(q4 + 1), q = __ldg(q4 + 2);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          float t, u, v;
          if (need[r] && alive[r] && id != self[r] && tri_hit<kGeo>(wr, light, o[r], op[r], a, b, q, t, u, v) &&
              t > kRayEps && t < t_max) {
            occluded[r] = true;
            alive[r] = false;
          }
        }
      }
    }
    if (st.sp == 0) break;
    --st.sp;
    entry = st.code[st.sp];
  }
  __syncwarp();
}

// sample_pixel_packet with R neighbouring sub-rays per lane (ss^2 a multiple
// of R).  The per-ray work, the order of the FP64 radiance and depth sums and
// the ray counts are those of the one-ray loop.
template <int kMode, int R, int kGeo = kGeoReference>
__device__ PixelSample sample_pixel_group(const SceneView &S, int pixel, bool active, const CellPose &pose,
                                          int *stack_code, float *stack_t, const SubraySample *subrays) {
  PixelSample out{0.0, -1.0f, true, 0u, 0u};
  double depth = 0;
  int valid_depth = 0;
  const float3 light = f3(pose.lx, pose.ly, pose.lz);
  const float3 origin = f3(pose.px, pose.py, pose.pz);
  const int ss = S.samples, n_sub = ss * ss;
  const int px_i = pixel % S.width, py_i = pixel / S.width;
  const HapkeConst hc = hapke_const(S.hapke);
  // hapke_directional_reflectance normalizes the light for every shaded ray
  // (hapke.hpp:153-157); it is the same vector for all of this lane's rays
  const float3 lnorm = normalize(light);
  const ShadowDir sdir = shadow_dir<kGeo>(light);
  for (int j = 0; j < n_sub; j += R) {
    float px[R], py[R];
    float3 ray[R], org[R];
    bool live[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (subrays) {
        px[r] = subrays[j + r].px;
        py[r] = subrays[j + r].py;
      } else {
        const int sx = (j + r) % ss, sy = (j + r) / ss;
        px[r] = subray_x(S, px_i, sx);
        py[r] = subray_y(S, py_i, sy);
      }
      ray[r] = normalize(rotate_ray(pose, f3(px[r], -py[r], -1)));
      org[r] = origin;
      live[r] = active && out.valid;
    }
    HitRecord hit[R];
    trace_nearest_packet_r<R, kGeo>(S, org, ray, live, stack_code, stack_t, hit);
    bool lit[R];
    float3 normal[R], sorigin[R];
    float albedo[R], r0[R];
    int self[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (active && out.valid) ++out.primary;
      if (hit[r].hit < 0) out.valid = false;
      const bool hitp = active && out.valid && hit[r].hit == 1;
      lit[r] = false;
      normal[r] = f3(0, 0, 0);
      sorigin[r] = f3(0, 0, 0);
      albedo[r] = S.hapke.w;
      r0[r] = hc.r0_w;
      self[r] = hit[r].tri;
      if (hitp) {
        if (kMode != kRadiance) {
          depth += hit[r].t;
          ++valid_depth;
        }
        if (kMode != kDepthOnly) {
          const float4 *q = reinterpret_cast<const float4 *>(S.shade + hit[r].tri);
          const float4 s0 = __ldg(q), s1 = __ldg(q + 1), s2 = __ldg(q + 2);
          const float w = 1 - hit[r].u - hit[r].v;
          normal[r] = normalize(f3(s0.x, s0.y, s0.z) * w + f3(s1.x, s1.y, s1.z) * hit[r].u +
                                f3(s2.x, s2.y, s2.z) * hit[r].v);
          lit[r] = !(dot(normal[r], light) <= 0 || dot(normal[r], -ray[r]) <= 0);
          if (lit[r]) {
            const float4 *t4 = tri_record<kGeo>(S, hit[r].tri, 2);
            const float4 a = __ldg(t4), b = __ldg(t4 + 1), c = __ldg(t4 + 2);
            sorigin[r] = shadow_origin_rec<kGeo>(a, b, c, hit[r].u, hit[r].v, light);
            if (S.has_albedo) {
              albedo[r] = s0.w * w + s1.w * hit[r].u + s2.w * hit[r].v;
              r0[r] = hfunc_r0(albedo[r]);
            }
          }
        }
      }
    }
    if (kMode != kDepthOnly) {
      bool any_lit = false;
#pragma unroll
      for (int r = 0; r < R; ++r) any_lit = any_lit || lit[r];
      if (__any_sync(kFull, any_lit)) {
        bool occ[R];
        trace_shadow_packet_r<R, kGeo>(S, sorigin, light, sdir, lit, self, stack_code, stack_t, occ);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (lit[r]) ++out.shadow;
          if (lit[r] && !occ[r]) {
            const double cos4 = subrays ? subrays[j + r].cos4 : cos4_of(px[r], py[r]);
            const float3 n = normalize(normal[r]), l = lnorm, v = normalize(-ray[r]);
            const float n_h = hapke_reflectance(dot(n, l), dot(n, v), dot(l, v), albedo[r], r0[r], S.hapke, hc);
            out.radiance += fmaxf(0, n_h * pose.intensity) * cos4;
          }
        }
      }
    }
  }
  out.radiance /= ss * ss;
  out.depth = valid_depth ? float(depth / valid_depth) : -1.0f;
  return out;
}

// One pixel at one pose sampled by a whole warp (sub-ray packets): the lanes
// carry the pixel's sub-rays, two each, so a packet spans one pixel's
// footprint -- the coherent shape when a pixel is wanted at only a few times
// (camera frames, the initial pose, adaptive probes).  Lane 0 forms the FP64
// radiance and depth sums in sub-ray order through shuffles, so the result is
// the same double as the serial loop of sample_pixel_packet.  Called by all
// 32 lanes with warp-uniform arguments; the result is valid in lane 0.
template <int kMode, int kGeo = kGeoReference>
__device__ PixelSample sample_pixel_subrays(const SceneView &S, int pixel, const CellPose &pose, int *stack_code,
                                            float *stack_t) {
  constexpr int R = 2;
  const int lane = threadIdx.x & 31;
  PixelSample out{0.0, -1.0f, true, 0u, 0u};
  double depth = 0;
  int valid_depth = 0;
  const float3 light = f3(pose.lx, pose.ly, pose.lz);
  const float3 origin = f3(pose.px, pose.py, pose.pz);
  const int ss = S.samples, n_sub = ss * ss;
  const int px_i = pixel % S.width, py_i = pixel / S.width;
  const HapkeConst hc = hapke_const(S.hapke);
  const float3 lnorm = normalize(light);  // as in sample_pixel_group
  const ShadowDir sdir = shadow_dir<kGeo>(light);
  bool valid = true;
  for (int g = 0; g < n_sub; g += 32 * R) {
    float px[R], py[R];
    float3 ray[R], org[R];
    bool live[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int j = g + lane * R + r;
      live[r] = valid && j < n_sub;
      const int jj = j < n_sub ? j : 0;
      px[r] = subray_x(S, px_i, jj % ss);
      py[r] = subray_y(S, py_i, jj / ss);
      ray[r] = normalize(rotate_ray(pose, f3(px[r], -py[r], -1)));
      org[r] = origin;
    }
    HitRecord hit[R];
    trace_nearest_packet_r<R, kGeo>(S, org, ray, live, stack_code, stack_t, hit);
    bool ovf = false, lit[R], hitp[R];
    float3 normal[R], sorigin[R];
    float albedo[R], r0[R];
    int self[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ovf = ovf || (live[r] && hit[r].hit < 0);
      hitp[r] = live[r] && hit[r].hit == 1;
      lit[r] = false;
      normal[r] = f3(0, 0, 0);
      sorigin[r] = f3(0, 0, 0);
      albedo[r] = S.hapke.w;
      r0[r] = hc.r0_w;
      self[r] = hit[r].tri;
      if (hitp[r] && kMode != kDepthOnly) {
        const float4 *q = reinterpret_cast<const float4 *>(S.shade + hit[r].tri);
        const float4 s0 = __ldg(q), s1 = __ldg(q + 1), s2 = __ldg(q + 2);
        const float w = 1 - hit[r].u - hit[r].v;
        normal[r] = normalize(f3(s0.x, s0.y, s0.z) * w + f3(s1.x, s1.y, s1.z) * hit[r].u +
                              f3(s2.x, s2.y, s2.z) * hit[r].v);
        lit[r] = !(dot(normal[r], light) <= 0 || dot(normal[r], -ray[r]) <= 0);
        if (lit[r]) {
          const float4 *t4 = tri_record<kGeo>(S, hit[r].tri, 2);
          const float4 a = __ldg(t4), b = __ldg(t4 + 1), c = __ldg(t4 + 2);
          sorigin[r] = shadow_origin_rec<kGeo>(a, b, c, hit[r].u, hit[r].v, light);
          if (S.has_albedo) {
            albedo[r] = s0.w * w + s1.w * hit[r].u + s2.w * hit[r].v;
            r0[r] = hfunc_r0(albedo[r]);
          }
        }
      }
    }
    double term[R] = {0.0, 0.0};
    if (kMode != kDepthOnly && __any_sync(kFull, lit[0] || lit[1])) {
      bool occ[R];
      trace_shadow_packet_r<R, kGeo>(S, sorigin, light, sdir, lit, self, stack_code, stack_t, occ);
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (lit[r] && !occ[r]) {
          const double cos4 = cos4_of(px[r], py[r]);
          const float3 n = normalize(normal[r]), l = lnorm, v = normalize(-ray[r]);
          const float n_h = hapke_reflectance(dot(n, l), dot(n, v), dot(l, v), albedo[r], r0[r], S.hapke, hc);
          term[r] = fmaxf(0, n_h * pose.intensity) * cos4;
        }
    }
    out.primary += __popc(__ballot_sync(kFull, live[0])) + __popc(__ballot_sync(kFull, live[1]));
    out.shadow += __popc(__ballot_sync(kFull, lit[0])) + __popc(__ballot_sync(kFull, lit[1]));
    // sums in sub-ray order j = g + src * R + r, formed by lane 0
    for (int src = 0; src < 32; ++src)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const double tv = __shfl_sync(kFull, term[r], src);
        const float dv = __shfl_sync(kFull, hit[r].t, src);
        const bool hv = __shfl_sync(kFull, hitp[r] ? 1 : 0, src) != 0;
        if (lane == 0) {
          out.radiance += tv;
          if (kMode != kRadiance && hv) {
            depth += dv;
            ++valid_depth;
          }
        }
      }
    if (__any_sync(kFull, ovf)) valid = false;
  }
  out.valid = valid;
  out.radiance /= ss * ss;
  out.depth = valid_depth ? float(depth / valid_depth) : -1.0f;
  return out;
}

__device__ __forceinline__ unsigned warp_sum(unsigned v) { return __reduce_add_sync(kFull, v); }

}  // namespace
}  // namespace dvsgb
