/*
 * CPU oracle for the DVS hot path -- TEST INFRASTRUCTURE ONLY (see
 * dvs_oracle.h).  A plain-C restatement of the reference algorithm of
 * BugBubbles/DvsRender4DeepSpace; every function cites the reference
 * file:line it follows.  Compiled with -ffp-contract=off; define ORACLE_FP64
 * for the FP64 variant of the geometry, ray and Hapke arithmetic.
 */
#include "dvs_oracle.h"
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_FP64
typedef double real;
#define R(x) (x)
#define REAL_EPS_HALF 1.1102230246251565e-16 /* 2^-53 */
#else
typedef float real;
#define R(x) (x##f)
#define REAL_EPS_HALF 5.960464477539063e-8f /* 2^-24, device_optics.cuh:42 */
#endif

/* kPi (include/dvs/math_types.hpp:37); the FP64 variant uses the double pi. */
#ifdef ORACLE_FP64
static const real kPi = 3.14159265358979323846;
#else
static const real kPi = 3.14159265358979323846f;
#endif
/* kRayEps and kMaxStackSize (include/helper_math.hpp:12-13). */
static const real kRayEps = R(1e-6);
#define kMaxStackSize 128

double oracle_pi_f32(void) { return (double)3.14159265358979323846f; }
int oracle_is_fp64(void) {
#ifdef ORACLE_FP64
  return 1;
#else
  return 0;
#endif
}

/* ---- small vector algebra (include/helper_math.hpp:18-77) ---------------- */
typedef struct { real x, y, z; } rv3;
static inline rv3 mk(real x, real y, real z) { rv3 r = {x, y, z}; return r; }
static inline rv3 from_f3(of3 a) { return mk((real)a.x, (real)a.y, (real)a.z); }
static inline rv3 add3(rv3 a, rv3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline rv3 sub3(rv3 a, rv3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline rv3 neg3(rv3 a) { return mk(-a.x, -a.y, -a.z); }
static inline rv3 scale3(real s, rv3 a) { return mk(a.x * s, a.y * s, a.z * s); }
static inline rv3 div3(rv3 a, real s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline real dot3(rv3 a, rv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline rv3 cross3(rv3 a, rv3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline rv3 normalize3(rv3 v) {
  real len = sqrt(dot3(v, v));
  if (len > R(0.0)) return div3(v, len);
  return mk(R(0.0), R(0.0), R(0.0));
}
static inline real clampr(real x, real lo, real hi) { return fmin(fmax(x, lo), hi); }

/* ---- Hapke (include/dvs/hapke.hpp:14-157) -------------------------------- */
typedef struct { real mu0, mue, S; } rough_terms;

static real safe_tan(real x) {  /* hapke.hpp:14-16 */
  return tan(clampr(x, -kPi / R(2.0) + R(1e-6), kPi / R(2.0) - R(1e-6)));
}
static real safe_acos(real x) { return acos(clampr(x, R(-1.0), R(1.0))); } /* :18-20 */
static real hg_double_lobe(real cosg, real b, real c) {                    /* :22-29 */
  const real one_minus_bb = R(1.0) - b * b;
  const real term1 = ((R(1.0) + c) * R(0.5)) * one_minus_bb /
                     pow(R(1.0) - R(2.0) * b * cosg + b * b, R(1.5));
  const real term2 = ((R(1.0) - c) * R(0.5)) * one_minus_bb /
                     pow(R(1.0) + R(2.0) * b * cosg + b * b, R(1.5));
  return term1 + term2;
}
static real b_s(real tan_g_div_2, real h_s) { /* :31-34 */
  if (h_s <= R(0.0)) return tan_g_div_2 <= R(0.0) ? R(1.0) : R(0.0);
  return R(1.0) / (R(1.0) + tan_g_div_2 / h_s);
}
static real b_c(real tan_g_div_2, real h_c) { /* :36-43 */
  if (h_c <= R(0.0)) return tan_g_div_2 <= R(0.0) ? R(1.0) : R(0.0);
  const real T = tan_g_div_2 / h_c;
  if (T < R(1e-8)) return R(1.0);
  return (R(1.0) + (R(1.0) - exp(-T)) / T) / (R(2.0) * (R(1.0) + T) * (R(1.0) + T));
}
static real hfunc(real x, real w) { /* :45-51 */
  if (x <= R(1e-8)) return R(1.0);
  const real root = sqrt(fmax(R(0.0), R(1.0) - w));
  const real r0 = (R(1.0) - root) / (R(1.0) + root);
  const real term = r0 + (R(1.0) - R(2.0) * r0 * x) * R(0.5) * log(R(1.0) + R(1.0) / x);
  return R(1.0) / (R(1.0) - w * x * term);
}
static real porosity_k(real phi) { /* :53-57 */
  if (phi <= R(1e-8)) return R(1.0);
  const real p = R(1.209) * pow(phi, R(2.0) / R(3.0));
  return -log(R(1.0) - p) / p;
}
static real chi_f(real thetap) { /* :59-62 */
  const real t = tan(thetap);
  return R(1.0) / sqrt(R(1.0) + kPi * t * t);
}
static real e1_f(real thetap, real cosy, real siny) { /* :64-67 */
  const real safe_siny = fmax(siny, R(1e-6));
  return exp((R(-2.0) / kPi) * (R(1.0) / tan(thetap)) * cosy / safe_siny);
}
static real e2_f(real thetap, real cosy, real siny) { /* :69-73 */
  const real safe_siny = fmax(siny, R(1e-6));
  const real v = (R(1.0) / tan(thetap)) * cosy / safe_siny;
  return exp((R(-1.0) / kPi) * v * v);
}
static real eta_f(real thetap, real cosy, real siny) { /* :75-80 */
  const real ch = chi_f(thetap);
  const real e1 = e1_f(thetap, cosy, siny);
  const real e2 = e2_f(thetap, cosy, siny);
  return ch * (cosy + siny * tan(thetap) * e2 / (R(2.0) - e1));
}
static real f_psi(real psi) { return exp(R(-2.0) * tan(psi * R(0.5))); } /* :82-84 */

static rough_terms rough_s(real cosi, real cose, real sini, real sine, real psi, real thetap) {
  /* hapke.hpp:86-129 */
  rough_terms out;
  if (thetap <= R(1e-8)) { out.mu0 = cosi; out.mue = cose; out.S = R(1.0); return out; }
  const real ch = chi_f(thetap);
  const real tan_thetap = tan(thetap);
  const real sin_psi_half = sin(psi * R(0.5));
  const real s2 = sin_psi_half * sin_psi_half;
  if (cosi >= cose) {
    out.mu0 = ch * (cosi + sini * tan_thetap *
                               (cos(psi) * e2_f(thetap, cose, sine) + s2 * e2_f(thetap, cosi, sini)) /
                               (R(2.0) - e1_f(thetap, cose, sine) - (psi / kPi) * e1_f(thetap, cosi, sini)));
    out.mue = ch * (cose + sine * tan_thetap *
                               (e2_f(thetap, cose, sine) - s2 * e2_f(thetap, cosi, sini)) /
                               (R(2.0) - e1_f(thetap, cose, sine) - (psi / kPi) * e1_f(thetap, cosi, sini)));
    out.S = out.mue / eta_f(thetap, cose, sine) * cosi / eta_f(thetap, cosi, sini) * ch /
            (R(1.0) - f_psi(psi) + f_psi(psi) * ch * (cosi / eta_f(thetap, cosi, sini)));
  } else {
    out.mu0 = ch * (cosi + sini * tan_thetap *
                               (e2_f(thetap, cosi, sini) - s2 * e2_f(thetap, cose, sine)) /
                               (R(2.0) - e1_f(thetap, cosi, sini) - (psi / kPi) * e1_f(thetap, cose, sine)));
    out.mue = ch * (cose + sine * tan_thetap *
                               (cos(psi) * e2_f(thetap, cosi, sini) + s2 * e2_f(thetap, cose, sine)) /
                               (R(2.0) - e1_f(thetap, cosi, sini) - (psi / kPi) * e1_f(thetap, cose, sine)));
    out.S = out.mue / eta_f(thetap, cose, sine) * cosi / eta_f(thetap, cosi, sini) * ch /
            (R(1.0) - f_psi(psi) + f_psi(psi) * ch * (cose / eta_f(thetap, cose, sine)));
  }
  return out;
}

static real hapke_reflectance_r(real cosi, real cose, real cosg, real albedo, const ohapke *p) {
  /* hapke.hpp:131-151 */
  if (cosi <= 0 || cose <= 0) return 0;
  cosi = clampr(cosi, 0, 1); cose = clampr(cose, 0, 1); cosg = clampr(cosg, -1, 1);
  const real sini = sqrt(fmax(R(0.0), 1 - cosi * cosi)), sine = sqrt(fmax(R(0.0), 1 - cose * cose));
  const real tan_g_div_2 = safe_tan(safe_acos(cosg) * R(0.5));
  const real psi = safe_acos((cosg - cosi * cose) / (sini * sine + R(1e-6)));
  const real p_g = hg_double_lobe(cosg, (real)p->b, (real)p->c);
  const real BS = b_s(tan_g_div_2, (real)p->hS);
  const real BC = b_c(tan_g_div_2, (real)p->hC);
  const real K = porosity_k((real)p->phi);
  const rough_terms rst = rough_s(cosi, cose, sini, sine, psi, (real)p->thetap);
  const real M = hfunc(rst.mu0 / K, albedo) * hfunc(rst.mue / K, albedo) - R(1.0);
  const real LS = rst.mu0 / (rst.mu0 + rst.mue + R(1e-6));
  return (albedo / (R(4.0) * kPi)) * LS * K * (p_g * (R(1.0) + BS * (real)p->B_S0) + M) *
         (R(1.0) + BC * (real)p->B_C0) * rst.S;
}

/* ---- Hapke, identity form ------------------------------------------------
 * hapke_reflectance_r above is hapke.hpp:131-151 in the reference's own
 * operation order.  The CUDA kernels evaluate the same reflectance through
 * identities that are exact in real arithmetic:
 *   tan(acos(c) / 2) = sqrt((1 - c) / (1 + c)), capped at tan(pi/2 - 1e-6)
 *                      (safe_tan, hapke.hpp:14-16);
 *   sin^2(psi / 2)   = (1 - cos psi) / 2;  cos(psi) = cos psi;
 *   tan(psi / 2)     = sqrt((1 - cos psi) / (1 + cos psi)), and -inf at
 *                      cos psi = -1, where the reference's tan(pi_f / 2) is
 *                      negative and its exp overflows (a NaN sample);
 *   y^1.5            = y * sqrt(y)  (hg_double_lobe, hapke.hpp:22-29);
 *   e1 = exp(-2/pi q), e2 = exp(-1/pi q^2) with one q = cot(thetap) cos y /
 *                      max(sin y, 1e-6)  (hapke.hpp:64-73).
 * hapke_reflectance_id_r restates that form in the kernels' operation order
 * (material constants hoisted as the kernels do, same values), so the
 * kernels' radiance is compared with it up to the ulps of acos/exp/log.  The
 * reference form stays the pinned one (golden vectors of hapke.hpp), and the
 * tests bound both forms against the FP64 oracle. */
static real pow15_r(real y) { return y * sqrt(y); }
static real hapke_reflectance_id_r(real cosi, real cose, real cosg, real albedo, const ohapke *p) {
  if (cosi <= 0 || cose <= 0) return 0;
  cosi = clampr(cosi, 0, 1); cose = clampr(cose, 0, 1); cosg = clampr(cosg, -1, 1);
  const real sini = sqrt(fmax(R(0.0), 1 - cosi * cosi)), sine = sqrt(fmax(R(0.0), 1 - cose * cose));
  const real tg_max = tan(kPi / R(2.0) - R(1e-6));
  const real tg = fmin(sqrt((R(1.0) - cosg) / (R(1.0) + cosg)), tg_max);
  const real cpsi = clampr((cosg - cosi * cose) / (sini * sine + R(1e-6)), R(-1.0), R(1.0));
  const real psi = acos(cpsi);
  const real b = (real)p->b, c = (real)p->c;
  const real one_minus_bb = R(1.0) - b * b;
  const real p_g = ((R(1.0) + c) * R(0.5)) * one_minus_bb / pow15_r(R(1.0) - R(2.0) * b * cosg + b * b) +
                   ((R(1.0) - c) * R(0.5)) * one_minus_bb / pow15_r(R(1.0) + R(2.0) * b * cosg + b * b);
  const real BS = b_s(tg, (real)p->hS);
  const real BC = (real)p->B_C0 != R(0.0) ? b_c(tg, (real)p->hC) : R(0.0);
  const real K = porosity_k((real)p->phi);
  real mu0, mue, S;
  if ((real)p->thetap <= R(1e-8)) {
    mu0 = cosi; mue = cose; S = R(1.0);
  } else {
    const real tan_thetap = tan((real)p->thetap);
    const real cot_t = R(1.0) / tan_thetap;
    const real ch = R(1.0) / sqrt(R(1.0) + kPi * tan_thetap * tan_thetap);
    const real s2 = (R(1.0) - cpsi) * R(0.5);
    const real qe = cot_t * cose / fmax(sine, R(1e-6)), qi = cot_t * cosi / fmax(sini, R(1e-6));
    const real e2e = exp((R(-1.0) / kPi) * qe * qe), e2i = exp((R(-1.0) / kPi) * qi * qi);
    const real e1e = exp((R(-2.0) / kPi) * qe), e1i = exp((R(-2.0) / kPi) * qi);
    const real eta_e = ch * (cose + sine * tan_thetap * e2e / (R(2.0) - e1e));
    const real eta_i = ch * (cosi + sini * tan_thetap * e2i / (R(2.0) - e1i));
#ifdef ORACLE_FP64
    /* pi_d / 2 < pi / 2: the reference's tan(psi / 2) at psi = acos(-1) is
     * +huge and its exp underflows to 0, as sqrt(2 / 0) = +inf gives. */
    const real tpsi = sqrt((R(1.0) - cpsi) / (R(1.0) + cpsi));
#else
    const real tpsi = cpsi > R(-1.0) ? sqrt((R(1.0) - cpsi) / (R(1.0) + cpsi)) : -(real)INFINITY;
#endif
    const real fp = exp(R(-2.0) * tpsi);
    if (cosi >= cose) {
      mu0 = ch * (cosi + sini * tan_thetap * (cpsi * e2e + s2 * e2i) / (R(2.0) - e1e - (psi / kPi) * e1i));
      mue = ch * (cose + sine * tan_thetap * (e2e - s2 * e2i) / (R(2.0) - e1e - (psi / kPi) * e1i));
      S = mue / eta_e * cosi / eta_i * ch / (R(1.0) - fp + fp * ch * (cosi / eta_i));
    } else {
      mu0 = ch * (cosi + sini * tan_thetap * (e2i - s2 * e2e) / (R(2.0) - e1i - (psi / kPi) * e1e));
      mue = ch * (cose + sine * tan_thetap * (cpsi * e2i + s2 * e2e) / (R(2.0) - e1i - (psi / kPi) * e1e));
      S = mue / eta_e * cosi / eta_i * ch / (R(1.0) - fp + fp * ch * (cose / eta_e));
    }
  }
  const real M = hfunc(mu0 / K, albedo) * hfunc(mue / K, albedo) - R(1.0);
  const real LS = mu0 / (mu0 + mue + R(1e-6));
  return (albedo / (R(4.0) * kPi)) * LS * K * (p_g * (R(1.0) + BS * (real)p->B_S0) + M) *
         (R(1.0) + BC * (real)p->B_C0) * S;
}

/* Form of the sampler's Hapke: 1 = identity form (the FP32 oracle's default,
 * the kernels' arithmetic), 0 = the reference's order (the FP64 oracle's
 * default).  Set before sampling; read-only while the sampler runs. */
#ifdef ORACLE_FP64
static int g_hapke_form = 0;
#else
static int g_hapke_form = 1;
#endif
void oracle_set_hapke_form(int form) { g_hapke_form = form ? 1 : 0; }
int oracle_hapke_form(void) { return g_hapke_form; }

static real hapke_form_r(int form, real cosi, real cose, real cosg, real albedo, const ohapke *p) {
  return form ? hapke_reflectance_id_r(cosi, cose, cosg, albedo, p)
              : hapke_reflectance_r(cosi, cose, cosg, albedo, p);
}

static real hapke_directional_r(rv3 normal, rv3 light, rv3 view, real albedo, const ohapke *p) {
  /* hapke.hpp:153-157 */
  rv3 n = normalize3(normal), l = normalize3(light), v = normalize3(view);
  return hapke_form_r(g_hapke_form, dot3(n, l), dot3(n, v), dot3(l, v), albedo, p);
}

/* The reference form (pinned bit for bit against hapke.hpp). */
float oracle_hapke_reflectance(float cosi, float cose, float cosg, float albedo, const ohapke *p) {
  return (float)hapke_reflectance_r(cosi, cose, cosg, albedo, p);
}
/* Either form, in this library's precision, returned in double. */
double oracle_hapke_reflectance_form(int form, double cosi, double cose, double cosg, double albedo,
                                     const ohapke *p) {
  return (double)hapke_form_r(form, (real)cosi, (real)cose, (real)cosg, (real)albedo, p);
}
float oracle_hapke_directional(const float *n, const float *l, const float *v, float albedo,
                               const ohapke *p) {
  /* hapke.hpp:153-157 in the reference form (pinned against the reference). */
  rv3 nn = normalize3(mk(n[0], n[1], n[2])), ll = normalize3(mk(l[0], l[1], l[2])),
      vv = normalize3(mk(v[0], v[1], v[2]));
  return (float)hapke_reflectance_r(dot3(nn, ll), dot3(nn, vv), dot3(ll, vv), albedo, p);
}

/* ---- pixel circuit (include/dvs/pixel_model.hpp:18-102), always FP64 ------ */
static double receptor_log_at(double u, double rate, double dt, double charge) {
  /* pixel_model.hpp:18-26 */
  if (dt <= 0) return u;
  rate = fmax(0.0, rate);
  double x = exp(u);
  if (rate == 0) return u - log1p(x * dt / charge);
  double a = exp(-rate * dt / charge), b = -expm1(-rate * dt / charge);
  return -log(a / x + b / rate);
}
double oracle_receptor_log_at(double u, double rate, double dt, double charge) {
  return receptor_log_at(u, rate, dt, charge);
}
static double contrast_at(double u, double rate, double dt, double ref, const opixel_params *p) {
  /* pixel_model.hpp:27-30 */
  return receptor_log_at(u, rate, dt, p->charge_scale) - ref + p->reference_leak * dt;
}

/* advance_pixel (pixel_model.hpp:34-102).  The oracle's normal() returns 0,
 * the reference test generator's behaviour (tests/test_sensor.cu:10). */
static int advance_pixel(opixel_state *s, const opixel_params *p, double rate, double t0, double t1,
                         double *out_t, int32_t *out_p, int capacity) {
  if (t1 <= t0) return 0;
  int count = 0;
  double cursor = t0, u = s->receptor_log;
  const double normal_draw = 0.0;
  /* Guard: with reference_leak > 0 the extremum split can shrink towards
   * the 1e-15 floor while the receptor no longer changes in double, so the
   * reference loop advances by ~1e-14 s per pass (a Zeno stall that takes
   * ~1e12 passes).  The oracle reports -2 after 2^20 passes instead. */
  long passes = 0;
  while (cursor < t1) {
    if (++passes > (1L << 20)) return -2;
    if (cursor < s->refractory_until) {
      double end = fmin(t1, s->refractory_until);
      u = receptor_log_at(u, rate, end - cursor, p->charge_scale);
      cursor = end;
      s->reference_log = u;
      if (cursor < t1 || cursor == s->refractory_until) {
        if (cursor >= s->refractory_until && s->reset_pending) {
          if (p->reset_noise_std > 0) s->reference_log += p->reset_noise_std * normal_draw;
          s->reset_pending = 0;
        }
      }
      if (cursor >= t1) break;
    } else if (s->reset_pending) {
      if (p->reset_noise_std > 0) s->reference_log += p->reset_noise_std * normal_draw;
      s->reset_pending = 0;
    }
    double remaining = t1 - cursor;
    double c0 = u - s->reference_log;
    double boundary = remaining;
    double x = exp(u), target = rate + p->charge_scale * p->reference_leak;
    if (p->reference_leak > 0 && x > target && target > rate) {
      double extremum;
      if (rate > 0)
        extremum = -p->charge_scale / rate * log((1.0 / target - 1.0 / rate) / (1.0 / x - 1.0 / rate));
      else
        extremum = p->charge_scale * (1.0 / target - 1.0 / x);
      if (extremum > 1e-15 && extremum < boundary) boundary = extremum;
    }
    double ub = receptor_log_at(u, rate, boundary, p->charge_scale);
    double cb = ub - s->reference_log + p->reference_leak * boundary;
    int polarity = -1;
    double level = 0;
    if (c0 >= s->threshold_pos) { polarity = 1; level = s->threshold_pos; }
    else if (c0 <= -s->threshold_neg) { polarity = 0; level = -s->threshold_neg; }
    else if (cb >= s->threshold_pos) { polarity = 1; level = s->threshold_pos; }
    else if (cb <= -s->threshold_neg) { polarity = 0; level = -s->threshold_neg; }
    if (polarity < 0) {
      u = ub;
      s->reference_log -= p->reference_leak * boundary;
      cursor += boundary;
      continue;
    }
    if (count == capacity) return -1;
    double lo = 0, hi = boundary;
    if (c0 >= s->threshold_pos || c0 <= -s->threshold_neg) hi = 0;
    else if (p->reference_leak == 0) {
      double target_inverse = exp(-(s->reference_log + level));
      double initial_inverse = exp(-u);
      if (rate > 0) {
        double stationary_inverse = 1.0 / rate;
        hi = -p->charge_scale / rate *
             log1p((target_inverse - initial_inverse) / (initial_inverse - stationary_inverse));
      } else
        hi = p->charge_scale * (target_inverse - initial_inverse);
      hi = fmin(boundary, fmax(0.0, hi));
    } else
      for (int j = 0; j < 48; ++j) {
        double mid = (lo + hi) * .5, c = contrast_at(u, rate, mid, s->reference_log, p);
        if (polarity ? c >= level : c <= level) hi = mid; else lo = mid;
      }
    u = receptor_log_at(u, rate, hi, p->charge_scale);
    cursor += hi;
    out_t[count] = cursor;
    out_p[count] = polarity;
    ++count;
    s->reference_log = u;
    s->refractory_until = cursor + p->refractory_time;
    s->reset_pending = 1;
  }
  s->receptor_log = u;
  return count;
}

int oracle_advance_pixel(opixel_state *s, const opixel_params *p, double rate, double t0, double t1,
                         double *event_t, int32_t *event_p, int capacity) {
  return advance_pixel(s, p, rate, t0, t1, event_t, event_p, capacity);
}

/* parameters() and photo_parameters() (src/cuda/event_sensor.cu:151-176). */
void oracle_derive_parameters(const ophysic *c, int physic_effects, opixel_params *p, ophoto *photo) {
  const double q = 1.602176634e-19, k = 1.380649e-23, h = 6.62607015e-34, cl = 299792458;
  p->threshold_pos = c->threshold_pos;
  p->threshold_neg = c->threshold_neg;
  double voltage = k * c->temperature_k / (q * c->subthreshold_kappa);
  p->charge_scale = c->receptor_capacitance_f * voltage / q;
  p->reference_leak = 0;
  p->reset_noise_std = 0;
  if (physic_effects) {
    p->refractory_time = c->refractory_time;
    p->reference_leak = c->reset_leakage_a / (c->reset_capacitance_f * voltage);
    p->reset_noise_std = c->reset_thermal_noise ? sqrt(k * c->temperature_k / c->reset_capacitance_f) / voltage : 0;
  } else {
    p->refractory_time = 0;
  }
  double pitch = c->pixel_pitch_um * 1e-6;
  float fnum2 = 4 * c->f_number * c->f_number; /* float arithmetic, event_sensor.cu:167 */
  photo->electrons_per_radiance = c->radiance_scale * 3.141592653589793 / fnum2 * c->lens_transmission *
                                  pitch * pitch * c->fill_factor * c->quantum_efficiency *
                                  (c->wavelength_nm * 1e-9) / (h * cl);
  photo->integration_step = c->circuit_step;
  if (physic_effects) {
    photo->dark_electrons = c->dark_current_a / q;
    photo->shot_noise = c->photon_shot_noise;
  } else {
    photo->dark_electrons = 0;
    photo->shot_noise = 0;
  }
}

/* ---- pose interpolation (include/dvs/device_optics.cuh:6-29) ------------- */
static float hermite(float a, float va, float b, float vb, float u, float dt) {
  float u2 = u * u, u3 = u2 * u;
  return a + (-2 * u3 + 3 * u2) * (b - a) + (u3 - 2 * u2 + u) * dt * va + (u3 - u2) * dt * vb;
}
static of3 hermite3(of3 a, of3 va, of3 b, of3 vb, float u, float dt) {
  of3 r = {hermite(a.x, va.x, b.x, vb.x, u, dt), hermite(a.y, va.y, b.y, vb.y, u, dt),
           hermite(a.z, va.z, b.z, vb.z, u, dt)};
  return r;
}
void oracle_optical_state_at(const ointerval *iv, double t, ostate *out) {
  /* device_optics.cuh:13-26 (pose state is float data in both variants) */
  float dt = (float)(iv->t1 - iv->t0);
  float u = dt > 0 ? (float)fmin(1.0, fmax(0.0, (t - iv->t0) / dt)) : 0;
  ostate s = iv->start;
  s.position = hermite3(iv->start.position, iv->start.velocity, iv->end.position, iv->end.velocity, u, dt);
  s.light = hermite3(iv->start.light, iv->start.light_rate, iv->end.light, iv->end.light_rate, u, dt);
  s.intensity = fmaxf(0.0f, hermite(iv->start.intensity, iv->start.intensity_rate, iv->end.intensity,
                                    iv->end.intensity_rate, u, dt));
  const float *a = iv->start.rotation;
  float b[4] = {iv->end.rotation[0], iv->end.rotation[1], iv->end.rotation[2], iv->end.rotation[3]};
  float d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
  if (d < 0) { b[0] = -b[0]; b[1] = -b[1]; b[2] = -b[2]; b[3] = -b[3]; d = -d; }
  float wa = 1 - u, wb = u;
  if (d < .9995f) {
    float angle = acosf(fminf(1, d)), inv = 1 / sinf(angle);
    wa = sinf((1 - u) * angle) * inv;
    wb = sinf(u * angle) * inv;
  }
  float q[4];
  for (int i = 0; i < 4; ++i) q[i] = wa * a[i] + wb * b[i];
  float norm = 1.0f / sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int i = 0; i < 4; ++i) s.rotation[i] = q[i] * norm;
  *out = s;
}
static rv3 rotate_ray(const float *q, rv3 v) { /* device_optics.cuh:27-29 */
  rv3 qv = mk(q[0], q[1], q[2]);
  rv3 c = scale3(R(2.0), cross3(qv, v));
  return add3(add3(v, scale3((real)q[3], c)), cross3(qv, c));
}

/* ---- BVH traversal (include/dvs/device_ray.hpp:6-158) --------------------- */
static rv3 inverse_direction(rv3 d) { /* device_ray.hpp:6-12 */
  rv3 inv;
  inv.x = R(1.0) / (fabs(d.x) > R(1e-20) ? d.x : copysign(R(1e-20), d.x));
  inv.y = R(1.0) / (fabs(d.y) > R(1e-20) ? d.y : copysign(R(1e-20), d.y));
  inv.z = R(1.0) / (fabs(d.z) > R(1e-20) ? d.z : copysign(R(1e-20), d.z));
  return inv;
}
static int intersect_two_children(rv3 P, rv3 idir, real t_min, real t_max, const obvh_node *bl,
                                  const obvh_node *br, real *dist) {
  /* device_ray.hpp:13-53 */
  real t1x0 = ((real)bl->bmin.x - P.x) * idir.x, t1x1 = ((real)bl->bmax.x - P.x) * idir.x;
  real t1y0 = ((real)bl->bmin.y - P.y) * idir.y, t1y1 = ((real)bl->bmax.y - P.y) * idir.y;
  real t1z0 = ((real)bl->bmin.z - P.z) * idir.z, t1z1 = ((real)bl->bmax.z - P.z) * idir.z;
  real t1min = fmax(fmax(fmin(t1x0, t1x1), fmin(t1y0, t1y1)), fmin(t1z0, t1z1));
  real t1max = fmin(fmin(fmax(t1x0, t1x1), fmax(t1y0, t1y1)), fmax(t1z0, t1z1));
  t1min = fmax(t_min, t1min);
  t1max = fmin(t_max, t1max);
  real t2x0 = ((real)br->bmin.x - P.x) * idir.x, t2x1 = ((real)br->bmax.x - P.x) * idir.x;
  real t2y0 = ((real)br->bmin.y - P.y) * idir.y, t2y1 = ((real)br->bmax.y - P.y) * idir.y;
  real t2z0 = ((real)br->bmin.z - P.z) * idir.z, t2z1 = ((real)br->bmax.z - P.z) * idir.z;
  real t2min = fmax(fmax(fmin(t2x0, t2x1), fmin(t2y0, t2y1)), fmin(t2z0, t2z1));
  real t2max = fmin(fmin(fmax(t2x0, t2x1), fmax(t2y0, t2y1)), fmax(t2z0, t2z1));
  t2min = fmax(t_min, t2min);
  t2max = fmin(t_max, t2max);
  dist[0] = t1min;
  dist[1] = t2min;
  int mask = 0;
  if (t1max >= t1min) mask |= 1;
  if (t2max >= t2min) mask |= 2;
  return mask;
}
static int intersect_triangle(rv3 ray, rv3 o, rv3 v0, rv3 v1, rv3 v2, real *out_t, real *out_u,
                              real *out_v) {
  /* Moller-Trumbore, device_ray.hpp:54-80 */
  const rv3 edge1 = sub3(v1, v0), edge2 = sub3(v2, v0);
  const rv3 pvec = cross3(ray, edge2);
  const real det = dot3(edge1, pvec);
  if (fabs(det) < kRayEps) return 0;
  const real inv_det = R(1.0) / det;
  const rv3 tvec = sub3(o, v0);
  const real u = dot3(tvec, pvec) * inv_det;
  if (u < R(0.0) || u > R(1.0)) return 0;
  const rv3 qvec = cross3(tvec, edge1);
  const real v = dot3(ray, qvec) * inv_det;
  if (v < R(0.0) || (u + v) > R(1.0)) return 0;
  const real t = dot3(edge2, qvec) * inv_det;
  if (t <= kRayEps) return 0;
  *out_t = t; *out_u = u; *out_v = v;
  return 1;
}
static inline rv3 vtx(const oscene *s, uint32_t i) { return from_f3(s->vertices[i]); }

typedef struct { int hit, tri; real t, u, v; } rhit;

/* Watertight ray/triangle test of the precision geometry (no reference
 * counterpart; the published algorithm of Woop, Benthin and Wald, "Watertight
 * Ray/Triangle Intersection", JCGT 2(1), 2013), in the operation order of the
 * CUDA kernels: shear onto +z along the dominant axis kz (kx/ky swapped when
 * the direction is negative there), 2-D edge functions U, V, W of the
 * projected vertices, an FP64 recomputation when one rounds to zero, all-same
 * signs for a hit; (u, v) = (V, W) / det in the reference's convention. */
typedef struct { int kx, ky, kz; real sx, sy, sz; } wt_ray;
static real comp3(rv3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static wt_ray wt_setup(rv3 d) {
  const real ax = fabs(d.x), ay = fabs(d.y), az = fabs(d.z);
  wt_ray w;
  w.kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  w.kx = w.kz == 2 ? 0 : w.kz + 1;
  w.ky = w.kx == 2 ? 0 : w.kx + 1;
  const real dz = comp3(d, w.kz);
  if (dz < R(0.0)) { const int k = w.kx; w.kx = w.ky; w.ky = k; }
  w.sx = comp3(d, w.kx) / dz;
  w.sy = comp3(d, w.ky) / dz;
  w.sz = R(1.0) / dz;
  return w;
}
static int intersect_watertight(const wt_ray *w, rv3 o, rv3 v0, rv3 v1, rv3 v2, real *out_t, real *out_u,
                                real *out_v) {
  const rv3 A = sub3(v0, o), B = sub3(v1, o), C = sub3(v2, o);
  const real az = comp3(A, w->kz), bz = comp3(B, w->kz), cz = comp3(C, w->kz);
  const real ax = comp3(A, w->kx) - w->sx * az, ay = comp3(A, w->ky) - w->sy * az;
  const real bx = comp3(B, w->kx) - w->sx * bz, by = comp3(B, w->ky) - w->sy * bz;
  const real cx = comp3(C, w->kx) - w->sx * cz, cy = comp3(C, w->ky) - w->sy * cz;
  real U = cx * by - cy * bx, V = ax * cy - ay * cx;
  /* opposite nonzero signs of U and V: a miss decided before W, as the kernels do */
  if ((U < R(0.0) && V > R(0.0)) || (U > R(0.0) && V < R(0.0))) return 0;
  real W = bx * ay - by * ax;
  if (U == R(0.0) || V == R(0.0) || W == R(0.0)) {
    U = (real)((double)cx * (double)by - (double)cy * (double)bx);
    V = (real)((double)ax * (double)cy - (double)ay * (double)cx);
    W = (real)((double)bx * (double)ay - (double)by * (double)ax);
  }
  if ((U < R(0.0) || V < R(0.0) || W < R(0.0)) && (U > R(0.0) || V > R(0.0) || W > R(0.0))) return 0;
  const real det = U + V + W;
  if (det == R(0.0)) return 0;
  const real T = U * (w->sz * az) + V * (w->sz * bz) + W * (w->sz * cz);
  const real rcp = R(1.0) / det;
  const real t = T * rcp;
  if (!(t > kRayEps)) return 0;
  *out_t = t; *out_u = V * rcp; *out_v = W * rcp;
  return 1;
}
/* The scene's triangle test: Moller-Trumbore or, in a precision scene, the
 * watertight test with the ray's shear w. */
static int scene_triangle(const oscene *s, const wt_ray *w, rv3 ray, rv3 o, rv3 v0, rv3 v1, rv3 v2, real *t,
                          real *u, real *v) {
  return s->watertight ? intersect_watertight(w, o, v0, v1, v2, t, u, v)
                       : intersect_triangle(ray, o, v0, v1, v2, t, u, v);
}

static rhit trace_nearest_r(const oscene *s, rv3 origin, rv3 ray) {
  /* device_ray.hpp:136-158 */
  rhit hit = {0, -1, 0, 0, 0};
  real closest = R(1e30);
  rv3 idir = inverse_direction(ray);
  const wt_ray w = wt_setup(ray);
  int stack[kMaxStackSize], sp = 0;
  stack[sp++] = s->root;
  while (sp > 0) {
    const obvh_node *node = &s->nodes[stack[--sp]];
    if (node->count > 0) {
      for (int i = 0; i < node->count; ++i) {
        int id = node->start + i;
        const uint32_t *tri = &s->indices[3 * (size_t)id];
        real t, u, v;
        if (scene_triangle(s, &w, ray, origin, vtx(s, tri[0]), vtx(s, tri[1]), vtx(s, tri[2]), &t, &u, &v) &&
            t < closest) {
          closest = t; hit.hit = 1; hit.tri = id; hit.t = t; hit.u = u; hit.v = v;
        }
      }
    } else {
      real dist[2];
      int mask = intersect_two_children(origin, idir, kRayEps, closest, &s->nodes[node->left],
                                        &s->nodes[node->right], dist);
      if (!mask) continue;
      if (sp + (mask == 3 ? 2 : 1) > kMaxStackSize) { hit.hit = -1; return hit; }
      if (mask == 3) {
        int left = dist[0] < dist[1];
        stack[sp++] = left ? node->right : node->left;
        stack[sp++] = left ? node->left : node->right;
      } else
        stack[sp++] = mask == 1 ? node->left : node->right;
    }
  }
  return hit;
}

static int trace_shadow_r(const oscene *s, rv3 origin, rv3 dir, int self, real t_min, real t_max) {
  /* trace_shadow_ray_any_hit, device_ray.hpp:81-135 */
  rv3 idir = inverse_direction(dir);
  const wt_ray w = wt_setup(dir);
  int stack[kMaxStackSize], sp = 0;
  stack[sp++] = s->root;
  while (sp > 0) {
    const obvh_node *node = &s->nodes[stack[--sp]];
    if (node->count > 0) {
      for (int i = 0; i < node->count; ++i) {
        int id = node->start + i;
        if (id == self) continue;
        const uint32_t *tri = &s->indices[3 * (size_t)id];
        real t, u, v;
        if (scene_triangle(s, &w, dir, origin, vtx(s, tri[0]), vtx(s, tri[1]), vtx(s, tri[2]), &t, &u, &v))
          if (t > t_min && t < t_max) return 1;
      }
      continue;
    }
    real dist[2];
    int mask = intersect_two_children(origin, idir, t_min, t_max, &s->nodes[node->left],
                                      &s->nodes[node->right], dist);
    if (mask == 0) continue;
    if (sp + (mask == 3 ? 2 : 1) > kMaxStackSize) return 1;
    if (mask == 3) {
      if (dist[0] < dist[1]) { stack[sp++] = node->right; stack[sp++] = node->left; }
      else { stack[sp++] = node->left; stack[sp++] = node->right; }
    } else if (mask == 1) stack[sp++] = node->left;
    else stack[sp++] = node->right;
  }
  return 0;
}

int oracle_trace_nearest(const oscene *s, const float *o, const float *d, int *tri, float *t, float *u,
                         float *v) {
  rhit h = trace_nearest_r(s, mk(o[0], o[1], o[2]), mk(d[0], d[1], d[2]));
  *tri = h.tri; *t = (float)h.t; *u = (float)h.u; *v = (float)h.v;
  return h.hit;
}
int oracle_trace_shadow(const oscene *s, const float *o, const float *d, int self) {
  return trace_shadow_r(s, mk(o[0], o[1], o[2]), mk(d[0], d[1], d[2]), self, kRayEps, R(1e30));
}

/* shadow_origin (device_optics.cuh:37-51); epsilon: the unit roundoff of its
 * error bound (the arithmetic's own: 2^-24 in FP32, 2^-53 in FP64). */
static rv3 shadow_origin_eps(const oscene *s, int tri_id, real u, real v, rv3 light, real epsilon) {
  const uint32_t *tri = &s->indices[3 * (size_t)tri_id];
  rv3 a = vtx(s, tri[0]), e1 = sub3(vtx(s, tri[1]), a), e2 = sub3(vtx(s, tri[2]), a);
  rv3 point = add3(add3(a, scale3(u, e1)), scale3(v, e2));
  rv3 normal = normalize3(cross3(e1, e2));
  if (dot3(normal, light) < 0) normal = neg3(normal);
  const real gamma = 8 * epsilon / (1 - 8 * epsilon);
  rv3 error = mk(gamma * (fabs(a.x) + fabs(u * e1.x) + fabs(v * e2.x)),
                 gamma * (fabs(a.y) + fabs(u * e1.y) + fabs(v * e2.y)),
                 gamma * (fabs(a.z) + fabs(u * e1.z) + fabs(v * e2.z)));
  real distance = fabs(normal.x) * error.x + fabs(normal.y) * error.y + fabs(normal.z) * error.z + R(1e-6);
  rv3 offset = scale3(distance, normal);
  point = add3(point, offset);
  const real inf = (real)INFINITY;
  if (offset.x != 0) point.x = nextafter(point.x, copysign(inf, offset.x));
  if (offset.y != 0) point.y = nextafter(point.y, copysign(inf, offset.y));
  if (offset.z != 0) point.z = nextafter(point.z, copysign(inf, offset.z));
  return point;
}
static rv3 shadow_origin_r(const oscene *s, int tri_id, real u, real v, rv3 light) {
  return shadow_origin_eps(s, tri_id, u, v, light, REAL_EPS_HALF);
}
void oracle_shadow_origin(const oscene *s, int tri, float u, float v, const float *light, float *out) {
  rv3 p = shadow_origin_r(s, tri, u, v, mk(light[0], light[1], light[2]));
  out[0] = (float)p.x; out[1] = (float)p.y; out[2] = (float)p.z;
}

static real material_albedo(real value, real fallback) { /* device_optics.cuh:30-33 */
  return isfinite(value) && value >= 0 && value <= 1 ? value : fallback;
}

/* Whether a lit sample can sit at Hapke's azimuth singularity in FP32: the
 * clamped ratio cos psi of hapke.hpp:96,123, evaluated in float arithmetic
 * from the sample's cosines moved by up to +-3e-7 (their FP32 error), reaches
 * -1 at a corner of that box.  There the reference's FP32 formula yields NaN
 * and the sample is dropped, while the FP64 value is finite; near-normal
 * views (sin e -> 0) make the ratio ill-conditioned. */
static int hapke_azimuth_singular(rv3 normal, rv3 light, rv3 view) {
  const rv3 n = normalize3(normal), l = normalize3(light), v = normalize3(view);
  const double ci = (double)dot3(n, l), ce = (double)dot3(n, v), cg = (double)dot3(l, v);
  for (int k = 0; k < 8; ++k) {
    float fi = (float)(ci + ((k & 1) ? 3e-7 : -3e-7)), fe = (float)(ce + ((k & 2) ? 3e-7 : -3e-7));
    float fg = (float)(cg + ((k & 4) ? 3e-7 : -3e-7));
    if (fi <= 0.0f || fe <= 0.0f) continue;
    fi = fminf(fmaxf(fi, 0.0f), 1.0f);
    fe = fminf(fmaxf(fe, 0.0f), 1.0f);
    fg = fminf(fmaxf(fg, -1.0f), 1.0f);
    const float si = sqrtf(fmaxf(0.0f, 1.0f - fi * fi)), se = sqrtf(fmaxf(0.0f, 1.0f - fe * fe));
    const float c = fminf(fmaxf((fg - fi * fe) / (si * se + 1e-6f), -1.0f), 1.0f);
    if (c <= -1.0f) return 1;
  }
  return 0;
}

/* One sub-ray of sample_pixel (device_optics.cuh:76-92): nearest hit,
 * shading test, shadow ray and Hapke term.  status: 1 hit, 0 miss, -1 stack
 * overflow; term: the sub-ray's radiance term (0 when unlit or shadowed);
 * cos4 is the sub-ray's field falloff. */
typedef struct { int status; real t; double term; int singular, crack; } osubray;

/* Whether a Moller-Trumbore hit lies within the FP32 rounding of its
 * barycentrics of an edge of the triangle: there an FP32 test of the same ray
 * can pass between this triangle and its neighbour across the edge (the test
 * is not watertight) and hit what lies behind.  The bound on each barycentric
 * is 16 * 2^-24 times the magnitudes of the dot product that forms it
 * (device_ray.hpp:62-75 operation order) over |det|. */
static int mt_crack(const oscene *s, rv3 o, rv3 d, int tri_id) {
  const uint32_t *tri = &s->indices[3 * (size_t)tri_id];
  const double u32 = 16 * 5.960464477539063e-8;
  const double v0[3] = {s->vertices[tri[0]].x, s->vertices[tri[0]].y, s->vertices[tri[0]].z};
  const double v1[3] = {s->vertices[tri[1]].x, s->vertices[tri[1]].y, s->vertices[tri[1]].z};
  const double v2[3] = {s->vertices[tri[2]].x, s->vertices[tri[2]].y, s->vertices[tri[2]].z};
  const double dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  double e1[3], e2[3], tv[3];
  for (int k = 0; k < 3; ++k) { e1[k] = v1[k] - v0[k]; e2[k] = v2[k] - v0[k]; tv[k] = oo[k] - v0[k]; }
  const double pv[3] = {dd[1] * e2[2] - dd[2] * e2[1], dd[2] * e2[0] - dd[0] * e2[2], dd[0] * e2[1] - dd[1] * e2[0]};
  const double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
  const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if (det == 0) return 1;
  const double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) / det;
  const double v = (dd[0] * qv[0] + dd[1] * qv[1] + dd[2] * qv[2]) / det;
  const double bu = u32 * (fabs(tv[0] * pv[0]) + fabs(tv[1] * pv[1]) + fabs(tv[2] * pv[2])) / fabs(det);
  const double bv = u32 * (fabs(dd[0] * qv[0]) + fabs(dd[1] * qv[1]) + fabs(dd[2] * qv[2])) / fabs(det);
  return u < bu || v < bv || 1.0 - u - v < bu + bv;
}
static osubray subray_eps(const oscene *s, const ostate *pose, rv3 position, rv3 light, rv3 ray, double cos4,
                          uint64_t *n_primary, uint64_t *n_shadow, real offset_eps) {
  osubray o = {0, R(0.0), 0.0, 0, 0};
  const real w_default = (real)s->hapke.w;
  ++*n_primary;
  rhit hit = trace_nearest_r(s, position, ray);
  o.status = hit.hit;
  if (hit.hit != 1) return o;
  o.t = hit.t;
  if (!s->watertight) o.crack = mt_crack(s, position, ray, hit.tri);
  const uint32_t *tri = &s->indices[3 * (size_t)hit.tri];
  real w = R(1.0) - hit.u - hit.v;
  rv3 n0 = from_f3(s->normals[tri[0]]), n1 = from_f3(s->normals[tri[1]]), n2 = from_f3(s->normals[tri[2]]);
  rv3 normal = normalize3(add3(add3(scale3(w, n0), scale3(hit.u, n1)), scale3(hit.v, n2)));
  if (dot3(normal, light) <= 0 || dot3(normal, neg3(ray)) <= 0) return o;
  rv3 origin = shadow_origin_eps(s, hit.tri, hit.u, hit.v, light, offset_eps);
  ++*n_shadow;
  if (trace_shadow_r(s, origin, light, hit.tri, kRayEps, R(1e30))) return o;
  real albedo = s->albedos ? material_albedo(s->albedos[tri[0]], w_default) * w +
                                 material_albedo(s->albedos[tri[1]], w_default) * hit.u +
                                 material_albedo(s->albedos[tri[2]], w_default) * hit.v
                           : w_default;
  o.term = fmax(R(0.0), hapke_directional_r(normal, light, neg3(ray), albedo, &s->hapke) *
                            (real)pose->intensity) * cos4;
  o.singular = hapke_azimuth_singular(normal, light, neg3(ray));
  return o;
}
static osubray subray_r(const oscene *s, const ostate *pose, rv3 position, rv3 light, rv3 ray, double cos4,
                        uint64_t *n_primary, uint64_t *n_shadow) {
  return subray_eps(s, pose, position, light, ray, cos4, n_primary, n_shadow, REAL_EPS_HALF);
}

/* ---- margin classification (test infrastructure; no reference counterpart) --
 * A sub-ray is a margin sub-ray when its outcome is discontinuous within the
 * rounding of an FP32 evaluation: re-traced with its image-plane direction
 * moved by +-eta in x and in y (eta a few times the FP32 error of a ray
 * direction), one of the four re-traces changes its hit status, its hit
 * distance by more than 1e-3 (a silhouette), or its radiance term by more
 * than 1e-3 of the larger term (a shadow or terminator boundary); or its
 * shadow ray, started from the shadow origin that the FP32 form of
 * shadow_origin's error bound gives (epsilon 2^-24: an offset off the surface
 * hundreds of times the FP64 one), changes the term likewise.  Smooth
 * changes -- crossing the shared edge of two triangles of one surface, the
 * shading gradient -- stay far below those jumps.  A pixel with a margin
 * sub-ray is a margin pixel.  g_margin_eta == 0 turns the test off. */
static double g_margin_eta = 0.0, g_margin_eta_c = 2.384185791015625e-7; /* 4 * 2^-24 */
static double g_margin_cond_tol = 1e-5;
void oracle_set_margin_eta(double eta) { g_margin_eta = eta > 0 ? eta : 0.0; }
void oracle_set_conditioning(double eta_c, double tolerance) {
  g_margin_eta_c = eta_c > 0 ? eta_c : 0.0;
  g_margin_cond_tol = tolerance > 0 ? tolerance : 1e-5;
}
static int subray_jumps(const osubray *a, const osubray *b) {
  if (a->status != b->status) return 1;
  if (a->status == 1 && fabs((double)b->t - (double)a->t) > 1e-3 * fabs((double)a->t)) return 1;
  const double big = fmax(a->term, b->term);
  return big > 0 && fabs(a->term - b->term) > 1e-3 * big;
}

/* sample_pixel (device_optics.cuh:73-94), every sub-ray moved by (dx, dy)
 * in the image plane (0, 0: the pixel itself).  Counts the rays it traces.
 * With margin != NULL and the margin test on, *margin |= 1 for a sub-ray
 * that jumps (subray_jumps) or sits at Hapke's azimuth singularity. */
static void sample_pixel_shifted(const oscene *s, int pixel, const ostate *pose, real dx, real dy,
                                 double *radiance_out, float *depth_out, int *valid_out, uint64_t *n_primary,
                                 uint64_t *n_shadow, uint8_t *margin) {
  double radiance = 0, depth = 0;
  int valid_depth = 0;
  const rv3 light = normalize3(from_f3(pose->light));
  const rv3 position = from_f3(pose->position);
  const int ss = s->samples;
  const real eta = (real)g_margin_eta;
  for (int sy = 0; sy < ss; ++sy)
    for (int sx = 0; sx < ss; ++sx) {
      real px = ((real)(pixel % s->width) + (sx + R(.5)) / (real)ss - R(.5) - (real)s->cx) / (real)s->fx;
      real py = ((real)(pixel / s->width) + (sy + R(.5)) / (real)ss - R(.5) - (real)s->cy) / (real)s->fy;
      px += dx;
      py += dy;
      rv3 ray = normalize3(rotate_ray(pose->rotation, mk(px, -py, R(-1.0))));
      const double cos4 = 1.0 / ((1.0 + px * px + py * py) * (1.0 + px * px + py * py));
      const osubray o = subray_r(s, pose, position, light, ray, cos4, n_primary, n_shadow);
      if (o.status < 0) { *radiance_out = 0; *depth_out = -1; *valid_out = 0; return; }
      if (margin && eta > 0 && o.crack) *margin |= 16;
      if (margin && eta > 0 && !(*margin & 1)) {
        if (o.singular) *margin |= 1;
        for (int k = 0; k < 4 && !(*margin & 1); ++k) {
          const real qx = px + (k == 0 ? eta : (k == 1 ? -eta : R(0.0)));
          const real qy = py + (k == 2 ? eta : (k == 3 ? -eta : R(0.0)));
          const rv3 moved = normalize3(rotate_ray(pose->rotation, mk(qx, -qy, R(-1.0))));
          uint64_t a = 0, b = 0;
          const osubray p = subray_r(s, pose, position, light, moved, cos4, &a, &b);
          if (subray_jumps(&o, &p)) *margin |= 1;
        }
        if (!(*margin & 1) && REAL_EPS_HALF != 5.960464477539063e-8) {
          uint64_t a = 0, b = 0;
          const osubray p = subray_eps(s, pose, position, light, ray, cos4, &a, &b, (real)5.960464477539063e-8);
          if (subray_jumps(&o, &p)) *margin |= 1;
        }
      }
      if (o.status == 0) continue;
      depth += o.t;
      ++valid_depth;
      radiance += o.term;
    }
  radiance /= ss * ss;
  *radiance_out = radiance;
  *depth_out = valid_depth ? (float)(depth / valid_depth) : -1.0f;
  *valid_out = 1;
}
static void sample_pixel_m(const oscene *s, int pixel, const ostate *pose, double *radiance_out,
                           float *depth_out, int *valid_out, uint64_t *n_primary, uint64_t *n_shadow,
                           uint8_t *margin) {
  sample_pixel_shifted(s, pixel, pose, R(0.0), R(0.0), radiance_out, depth_out, valid_out, n_primary, n_shadow,
                       margin);
}
static void sample_pixel_r(const oscene *s, int pixel, const ostate *pose, double *radiance_out,
                           float *depth_out, int *valid_out, uint64_t *n_primary, uint64_t *n_shadow) {
  sample_pixel_m(s, pixel, pose, radiance_out, depth_out, valid_out, n_primary, n_shadow, NULL);
}

/* Conditioning class of a pixel: its radiance or depth, as this oracle
 * computes them, moves by more than `tolerance` (relative) when every
 * sub-ray is moved by +-eta_c in x or in y, eta_c about the FP32 error of a
 * ray direction.  Such a pixel's value is not fixed to the tolerance by a
 * float ray at all (grazing incidence with varying vertex normals, a shadow
 * edge or silhouette inside the pixel).  Returns 8 for a conditioning pixel. */
static uint8_t pixel_conditioning(const oscene *s, int pixel, const ostate *pose, double radiance, float depth,
                                  double eta_c, double tolerance) {
  for (int k = 0; k < 4; ++k) {
    const real dx = (real)(k == 0 ? eta_c : (k == 1 ? -eta_c : 0.0));
    const real dy = (real)(k == 2 ? eta_c : (k == 3 ? -eta_c : 0.0));
    double r;
    float d;
    int valid;
    uint64_t a = 0, b = 0;
    sample_pixel_shifted(s, pixel, pose, dx, dy, &r, &d, &valid, &a, &b, NULL);
    if (!valid) return 8;
    const double big = fmax(fabs(r), fabs(radiance));
    if (big > 0 && fabs(r - radiance) > tolerance * big) return 8;
    if ((d < 0) != (depth < 0)) return 8;
    if (depth > 0 && fabs((double)d - (double)depth) > tolerance * (double)depth) return 8;
  }
  return 0;
}

void oracle_sample_pixel(const oscene *s, int pixel, const ostate *pose, double *radiance, float *depth,
                         int *valid) {
  uint64_t a = 0, b = 0;
  sample_pixel_r(s, pixel, pose, radiance, depth, valid, &a, &b);
}

static int thread_count(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

void oracle_render(const oscene *s, const ostate *pose, double *radiance, float *depth, int *valid,
                   int nthreads) {
  const int n = s->width * s->height;
  const int nt = thread_count(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int i = 0; i < n; ++i) {
    uint64_t a = 0, b = 0;
    sample_pixel_r(s, i, pose, &radiance[i], &depth[i], &valid[i], &a, &b);
  }
}

void oracle_render_pixels(const oscene *s, const ostate *pose, const int32_t *pixels, int n,
                          double *radiance, float *depth, int nthreads, uint64_t *primary_rays,
                          uint64_t *shadow_rays) {
  const int nt = thread_count(nthreads);
  (void)nt;
  uint64_t prim = 0, shad = 0;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt) reduction(+ : prim, shad)
  for (int i = 0; i < n; ++i) {
    int valid;
    uint64_t a = 0, b = 0;
    sample_pixel_r(s, pixels[i], pose, &radiance[i], &depth[i], &valid, &a, &b);
    prim += a;
    shad += b;
  }
  *primary_rays = prim;
  *shadow_rays = shad;
}

void oracle_render_pixels_margin(const oscene *s, const ostate *pose, const int32_t *pixels, int n,
                                 double *radiance, float *depth, uint8_t *margin, int nthreads) {
  const int nt = thread_count(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
  for (int i = 0; i < n; ++i) {
    int valid;
    uint64_t a = 0, b = 0;
    margin[i] = 0;
    sample_pixel_m(s, pixels[i], pose, &radiance[i], &depth[i], &valid, &a, &b, &margin[i]);
    if (!valid) {
      radiance[i] = NAN;
      continue;
    }
    if (g_margin_eta > 0)
      margin[i] |= pixel_conditioning(s, pixels[i], pose, radiance[i], depth[i], g_margin_eta_c, g_margin_cond_tol);
  }
}

/* ---- BVH build (src/bvh/build.cpp, src/bvh/bining.cpp, include/bvh/common.h) */
typedef struct { of3 min, max; } oaabb;
typedef struct { oaabb bounds; of3 center; int tri_index; } oref;

static oaabb aabb_empty(void) { /* common.h:6-11 */
  oaabb b = {{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};
  return b;
}
static int aabb_is_empty(const oaabb *b) { /* common.h:13-16 */
  return (b->min.x > b->max.x) | (b->min.y > b->max.y) | (b->min.z > b->max.z);
}
static void aabb_grow_point(oaabb *b, of3 p) { /* common.h:18-26 */
  b->min.x = (p.x < b->min.x ? p.x : b->min.x);
  b->min.y = (p.y < b->min.y ? p.y : b->min.y);
  b->min.z = (p.z < b->min.z ? p.z : b->min.z);
  b->max.x = (p.x > b->max.x ? p.x : b->max.x);
  b->max.y = (p.y > b->max.y ? p.y : b->max.y);
  b->max.z = (p.z > b->max.z ? p.z : b->max.z);
}
static inline float mn(float a, float b) { return (b < a) ? b : a; } /* std::min */
static inline float mx(float a, float b) { return (a < b) ? b : a; } /* std::max */
static void aabb_grow_box(oaabb *b, const oaabb *o) { /* common.h:28-48 */
  if (aabb_is_empty(o)) return;
  float xmin = mn(o->min.x, o->max.x), ymin = mn(o->min.y, o->max.y), zmin = mn(o->min.z, o->max.z);
  float xmax = mx(o->min.x, o->max.x), ymax = mx(o->min.y, o->max.y), zmax = mx(o->min.z, o->max.z);
  b->min.x = mn(b->min.x, xmin); b->min.y = mn(b->min.y, ymin); b->min.z = mn(b->min.z, zmin);
  b->max.x = mx(b->max.x, xmax); b->max.y = mx(b->max.y, ymax); b->max.z = mx(b->max.z, zmax);
}
static of3 aabb_center(const oaabb *b) { /* common.h:50-52 */
  of3 c = {(b->min.x + b->max.x) * 0.5f, (b->min.y + b->max.y) * 0.5f, (b->min.z + b->max.z) * 0.5f};
  return c;
}
static float aabb_safe_area(const oaabb *b) { /* common.h:54-57 */
  float dx = b->max.x - b->min.x, dy = b->max.y - b->min.y, dz = b->max.z - b->min.z;
  return mx(dx * dy + dy * dz + dz * dx, 1e-12f);
}
static float f3get(of3 v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }

typedef struct {
  int max_leaf;
  oref *refs;
  obvh_node *nodes;
  int n_nodes;
} obuild;

static int create_leaf(obuild *ctx, int start, int end, const oaabb *box) { /* build.cpp:176-187 */
  obvh_node *n = &ctx->nodes[ctx->n_nodes];
  n->bmin = box->min; n->bmax = box->max;
  n->left = -1; n->right = -1; n->start = start; n->count = end - start;
  return ctx->n_nodes++;
}

#define NUM_BINS 32
static int build_node(obuild *ctx, int start, int end) { /* build.cpp:126-174 */
  int range_size = end - start;
  oaabb range_box = aabb_empty();
  for (int i = start; i < end; ++i) aabb_grow_box(&range_box, &ctx->refs[i].bounds);
  if (range_size <= ctx->max_leaf) return create_leaf(ctx, start, end, &range_box);

  /* BVHObjectBinning constructor (bining.cpp:9-98) */
  oref *refs = ctx->refs;
  oaabb cent = aabb_empty();
  for (int i = 0; i < range_size; ++i) aabb_grow_point(&cent, aabb_center(&refs[start + i].bounds));
  size_t nb_f = (size_t)(4.0f + 0.05f * (float)range_size);
  int num_bins = (int)(nb_f < (size_t)NUM_BINS ? nb_f : (size_t)NUM_BINS);
  float ext[3] = {cent.max.x - cent.min.x, cent.max.y - cent.min.y, cent.max.z - cent.min.z};
  float scale[3];
  for (int d = 0; d < 3; ++d) { ext[d] = fmaxf(ext[d], 1e-12f); scale[d] = (float)num_bins / ext[d]; }
  oaabb bins_b[3][NUM_BINS];
  int bins_c[3][NUM_BINS];
  for (int d = 0; d < 3; ++d)
    for (int b = 0; b < NUM_BINS; ++b) { bins_b[d][b] = aabb_empty(); bins_c[d][b] = 0; }
  for (int i = 0; i < range_size; ++i) {
    const oref *ref = &refs[start + i];
    int bin[3];
    for (int d = 0; d < 3; ++d) {
      int idx = (int)((f3get(ref->center, d) - f3get(cent.min, d)) * scale[d]);
      bin[d] = idx < 0 ? 0 : (idx > num_bins - 1 ? num_bins - 1 : idx);
    }
    for (int d = 0; d < 3; ++d) { aabb_grow_box(&bins_b[d][bin[d]], &ref->bounds); bins_c[d][bin[d]]++; }
  }
  float leaf_sah = aabb_safe_area(&range_box) * (float)range_size;
  float best_cost = FLT_MAX;
  int best_dim = 0, best_pos = 0;
  for (int d = 0; d < 3; ++d) {
    oaabb right_bounds[NUM_BINS];
    int right_count[NUM_BINS];
    oaabb cur = aabb_empty();
    int cnt = 0;
    for (int b = num_bins - 1; b >= 0; --b) {
      aabb_grow_box(&cur, &bins_b[d][b]);
      cnt += bins_c[d][b];
      right_bounds[b] = cur;
      right_count[b] = cnt;
    }
    oaabb lb = aabb_empty();
    int lc = 0;
    for (int b = 1; b < num_bins; ++b) {
      aabb_grow_box(&lb, &bins_b[d][b - 1]);
      lc += bins_c[d][b - 1];
      int rc = right_count[b];
      float cost = aabb_safe_area(&lb) * (float)lc + aabb_safe_area(&right_bounds[b]) * (float)rc;
      if (cost < best_cost) { best_cost = cost; best_dim = d; best_pos = b; }
    }
  }
  /* build.cpp:142-147 (sah costs are 1 in BVHBuildParams, build.h:9-13) */
  float leaf_cost = 1.0f * leaf_sah;
  float split_cost = 1.0f * aabb_safe_area(&range_box) + 1.0f * best_cost;
  if (leaf_cost <= split_cost) return create_leaf(ctx, start, end, &range_box);

  /* BVHObjectBinning::split (bining.cpp:110-182) */
  int l = start, r = end - 1;
  float cmin = f3get(cent.min, best_dim), cmax = f3get(cent.max, best_dim);
  float split_val = cmin + ((float)best_pos / (float)num_bins) * (cmax - cmin);
  while (l <= r) {
    if (f3get(refs[l].center, best_dim) < split_val) l++;
    else { oref tmp = refs[l]; refs[l] = refs[r]; refs[r] = tmp; r--; }
  }
  int mid = l;
  if (mid - start == 0 || end - mid == 0) mid = start + range_size / 2;
  int left_idx = build_node(ctx, start, mid);
  int right_idx = build_node(ctx, mid, end);
  obvh_node *n = &ctx->nodes[ctx->n_nodes];
  n->bmin = range_box.min; n->bmax = range_box.max;
  n->left = left_idx; n->right = right_idx; n->start = 0; n->count = 0;
  return ctx->n_nodes++;
}

int oracle_bvh_build(int max_leaf_size, const float *vertices, int n_vertices, uint32_t *indices,
                     int n_triangles, obvh_node *nodes, int *n_nodes) {
  /* BVHBuilder::build (build.cpp:27-76) */
  (void)n_vertices;
  *n_nodes = 0;
  if (n_triangles <= 0) return -1;
  obuild ctx;
  ctx.max_leaf = max_leaf_size;
  ctx.nodes = nodes;
  ctx.n_nodes = 0;
  ctx.refs = (oref *)malloc(sizeof(oref) * (size_t)n_triangles);
  if (!ctx.refs) return -1;
  const of3 *v = (const of3 *)vertices;
  for (int i = 0; i < n_triangles; ++i) {
    of3 a = v[indices[3 * (size_t)i]], b = v[indices[3 * (size_t)i + 1]], c = v[indices[3 * (size_t)i + 2]];
    oaabb box;
    box.min.x = fminf(fminf(a.x, b.x), c.x); box.min.y = fminf(fminf(a.y, b.y), c.y);
    box.min.z = fminf(fminf(a.z, b.z), c.z);
    box.max.x = fmaxf(fmaxf(a.x, b.x), c.x); box.max.y = fmaxf(fmaxf(a.y, b.y), c.y);
    box.max.z = fmaxf(fmaxf(a.z, b.z), c.z);
    ctx.refs[i].bounds = box;
    ctx.refs[i].center = aabb_center(&box);
    ctx.refs[i].tri_index = i;
  }
  int root = build_node(&ctx, 0, n_triangles);
  uint32_t *reordered = (uint32_t *)malloc(sizeof(uint32_t) * 3 * (size_t)n_triangles);
  for (int i = 0; i < n_triangles; ++i)
    memcpy(&reordered[3 * (size_t)i], &indices[3 * (size_t)ctx.refs[i].tri_index], 3 * sizeof(uint32_t));
  memcpy(indices, reordered, sizeof(uint32_t) * 3 * (size_t)n_triangles);
  free(reordered);
  free(ctx.refs);
  *n_nodes = ctx.n_nodes;
  return root;
}

int oracle_bvh_validate(const obvh_node *nodes, int n_nodes, int root) {
  /* BVHBuilder::validate (build.cpp:188-242) */
  if (root < 0 || root >= n_nodes) return -1;
  char *visited = (char *)calloc((size_t)n_nodes, 1);
  int *stack = (int *)malloc(sizeof(int) * (size_t)(n_nodes + 2));
  int sp = 0, status = 0;
  stack[sp++] = root;
  while (sp > 0) {
    int idx = stack[--sp];
    if (idx < 0 || idx >= n_nodes || visited[idx]) { status = -1; break; }
    visited[idx] = 1;
    const obvh_node *n = &nodes[idx];
    if (n->count > 0) {
      if (n->left != -1 || n->right != -1) { status = -1; break; }
      continue;
    }
    if (n->left < 0 || n->left >= n_nodes || n->right < 0 || n->right >= n_nodes) { status = -1; break; }
    if (sp + 2 > n_nodes + 2) { status = -1; break; }
    stack[sp++] = n->right;
    stack[sp++] = n->left;
  }
  free(stack);
  free(visited);
  return status;
}

/* ---- event readout FIFO (src/event_readout.cpp:6-34) -------------------- */
typedef struct { double ready_time; oevent event; } opending;
struct oreadout {
  double bandwidth, latency, available;
  size_t capacity, dropped, peak;
  opending *q;
  size_t q_cap, q_head, q_size;
};

oreadout *oracle_readout_create(double bandwidth, double latency, size_t capacity) {
  oreadout *r = (oreadout *)calloc(1, sizeof(oreadout));
  r->bandwidth = bandwidth; r->latency = latency; r->capacity = capacity;
  return r;
}
void oracle_readout_destroy(oreadout *r) {
  if (!r) return;
  free(r->q);
  free(r);
}
static void q_push(oreadout *r, opending p) {
  if (r->q_size == r->q_cap) {
    size_t nc = r->q_cap ? 2 * r->q_cap : 1024;
    opending *nq = (opending *)malloc(sizeof(opending) * nc);
    for (size_t i = 0; i < r->q_size; ++i) nq[i] = r->q[(r->q_head + i) % r->q_cap];
    free(r->q);
    r->q = nq; r->q_cap = nc; r->q_head = 0;
  }
  r->q[(r->q_head + r->q_size) % r->q_cap] = p;
  r->q_size++;
}
static opending *q_front(oreadout *r) { return &r->q[r->q_head]; }
static void q_pop(oreadout *r) { r->q_head = (r->q_head + 1) % r->q_cap; r->q_size--; }

static int event_less(const oevent *a, const oevent *b) { /* event_readout.cpp:8-12 */
  if (a->timestamp != b->timestamp) return a->timestamp < b->timestamp;
  if (a->y != b->y) return a->y < b->y;
  return a->x < b->x;
}
static void stable_sort_events(oevent *e, size_t n) { /* std::stable_sort: bottom-up merge */
  if (n < 2) return;
  oevent *tmp = (oevent *)malloc(sizeof(oevent) * n);
  for (size_t width = 1; width < n; width *= 2) {
    for (size_t lo = 0; lo < n; lo += 2 * width) {
      size_t mid = lo + width < n ? lo + width : n, hi = lo + 2 * width < n ? lo + 2 * width : n;
      size_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) tmp[k++] = event_less(&e[j], &e[i]) ? e[j++] : e[i++];
      while (i < mid) tmp[k++] = e[i++];
      while (j < hi) tmp[k++] = e[j++];
    }
    memcpy(e, tmp, sizeof(oevent) * n);
  }
  free(tmp);
}

int oracle_readout_submit(oreadout *r, const oevent *events_in, size_t n, double now, oevent *ready,
                          size_t ready_cap, size_t *n_ready) {
  size_t out = 0;
  int status = 0;
#define EMIT(ev) do { if (out < ready_cap) ready[out] = (ev); else status = 6; ++out; } while (0)
  oevent *events = (oevent *)malloc(sizeof(oevent) * (n ? n : 1));
  if (n) memcpy(events, events_in, sizeof(oevent) * n);
  stable_sort_events(events, n);
  for (size_t i = 0; i < n; ++i) {
    const oevent *e = &events[i];
    while (r->q_size && q_front(r)->ready_time <= e->timestamp) { EMIT(q_front(r)->event); q_pop(r); }
    if (r->bandwidth <= 0) { EMIT(*e); continue; }
    if (r->q_size >= r->capacity) { r->dropped++; continue; }
    double completed = fmax(r->available, e->timestamp) + 1.0 / r->bandwidth;
    r->available = completed;
    opending p;
    p.ready_time = completed + r->latency;
    p.event = *e;
    p.event.timestamp = completed + r->latency;
    q_push(r, p);
    if (r->q_size > r->peak) r->peak = r->q_size;
  }
  while (r->q_size && q_front(r)->ready_time <= now) { EMIT(q_front(r)->event); q_pop(r); }
  free(events);
  *n_ready = out;
  return status;
}
int oracle_readout_drain(oreadout *r, oevent *ready, size_t ready_cap, size_t *n_ready) {
  size_t out = 0;
  int status = 0;
  while (r->q_size) { EMIT(q_front(r)->event); q_pop(r); }
  *n_ready = out;
  return status;
#undef EMIT
}
size_t oracle_readout_dropped(const oreadout *r) { return r->dropped; }
size_t oracle_readout_peak(const oreadout *r) { return r->peak; }

/* ---- event sensor (src/cuda/event_sensor.cu:18-60,244-305) -------------- */
struct osensor {
  oscene scene;
  opixel_params params;
  ophoto photo;
  int max_events, initialized;
  double threshold_std, threshold_min, last_time;
  opixel_state *states;
  oreadout *readout;
  uint64_t primary_rays, shadow_rays;
  /* margin classification (oracle_sensor_set_margin): per pixel the flags
   * (1 optical margin at a cell sample, 2 circuit margin, 4 optical margin of
   * an event-time depth sample) and two shadow circuits with both thresholds
   * moved by +shift and -shift, whose polarity sequences are compared with the
   * circuit's own through a count and a running hash per circuit */
  int classify;
  double threshold_shift;
  uint8_t *margin;
  opixel_state *shifted;     /* 2 per pixel: +shift, -shift */
  uint64_t *seq;             /* 3 per pixel: (count << 48) ^ hash of the polarity sequence */
};

static void seq_push(uint64_t *seq, const int32_t *pol, int n) {
  uint64_t count = *seq >> 48, hash = *seq & 0xffffffffffffull;
  for (int j = 0; j < n; ++j) {
    hash = (hash * 3 + (uint64_t)(pol[j] + 1)) & 0xffffffffffffull;
    ++count;
  }
  *seq = (count << 48) | hash;
}

osensor *oracle_sensor_create(const oscene *scene, const ophysic *c, int physic_effects, int aer_delay) {
  /* EventSensor::EventSensor (event_sensor.cu:244-260) */
  int n = scene->width * scene->height;
  if (scene->width <= 0 || scene->height <= 0 || c->max_events_per_step < 1 || c->max_events_per_step > 64)
    return NULL;
  osensor *s = (osensor *)calloc(1, sizeof(osensor));
  s->scene = *scene;
  oracle_derive_parameters(c, physic_effects, &s->params, &s->photo);
  s->max_events = c->max_events_per_step;
  s->threshold_std = physic_effects ? c->threshold_std : 0;
  s->threshold_min = c->threshold_min;
  s->states = (opixel_state *)calloc((size_t)n, sizeof(opixel_state));
  s->readout = oracle_readout_create(aer_delay ? (double)c->readout_bandwidth : 0,
                                     aer_delay ? (double)c->readout_latency : 0,
                                     (size_t)c->readout_queue_capacity);
  return s;
}
int oracle_sensor_set_margin(osensor *s, double threshold_shift) {
  /* before initialize: the shadow circuits start from the same state */
  if (s->initialized || !(threshold_shift > 0)) return 3;
  const size_t n = (size_t)s->scene.width * s->scene.height;
  s->classify = 1;
  s->threshold_shift = threshold_shift;
  s->margin = (uint8_t *)calloc(n, 1);
  s->shifted = (opixel_state *)calloc(2 * n, sizeof(opixel_state));
  s->seq = (uint64_t *)calloc(3 * n, sizeof(uint64_t));
  return 0;
}
void oracle_sensor_margins(const osensor *s, uint8_t *out) {
  const size_t n = (size_t)s->scene.width * s->scene.height;
  for (size_t i = 0; i < n; ++i) {
    uint8_t m = s->classify ? s->margin[i] : 0;
    if (s->classify && (s->seq[3 * i] != s->seq[3 * i + 1] || s->seq[3 * i] != s->seq[3 * i + 2])) m |= 2;
    out[i] = m;
  }
}
void oracle_sensor_destroy(osensor *s) {
  if (!s) return;
  free(s->margin);
  free(s->shifted);
  free(s->seq);
  free(s->states);
  oracle_readout_destroy(s->readout);
  free(s);
}

int oracle_sensor_initialize(osensor *s, const ostate *pose, double t, int nthreads) {
  /* EventSensor::initialize + initialize_pixels (event_sensor.cu:18-28,262-270) */
  if (!isfinite(t) || s->initialized) return 3;
  if (s->threshold_std != 0 || s->photo.shot_noise || s->params.reset_noise_std != 0) return 3;
  const int n = s->scene.width * s->scene.height;
  int error = 0;
  const int nt = thread_count(nthreads);
  (void)nt;
  uint64_t prim = 0, shad = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt) reduction(+ : prim, shad)
  for (int i = 0; i < n; ++i) {
    double rad;
    float depth;
    int valid;
    uint64_t a = 0, b = 0;
    sample_pixel_m(&s->scene, i, pose, &rad, &depth, &valid, &a, &b, s->classify ? &s->margin[i] : NULL);
    prim += a;
    shad += b;
    if (!valid || !isfinite(rad)) {
#pragma omp atomic write
      error = 2;
      continue;
    }
    opixel_state st;
    st.receptor_log = st.reference_log =
        log(fmax(1e-30, rad * s->photo.electrons_per_radiance + s->photo.dark_electrons));
    st.refractory_until = -1;
    st.reset_pending = 0;
    /* threshold mismatch draws are zero in the deterministic oracle */
    st.threshold_pos = fmax(s->threshold_min, s->params.threshold_pos + s->threshold_std * 0.0);
    st.threshold_neg = fmax(s->threshold_min, s->params.threshold_neg + s->threshold_std * 0.0);
    s->states[i] = st;
    if (s->classify) {
      opixel_state hi = st, lo = st;
      hi.threshold_pos += s->threshold_shift;
      hi.threshold_neg += s->threshold_shift;
      lo.threshold_pos -= s->threshold_shift;
      lo.threshold_neg -= s->threshold_shift;
      s->shifted[2 * (size_t)i] = hi;
      s->shifted[2 * (size_t)i + 1] = lo;
    }
  }
  s->primary_rays += prim;
  s->shadow_rays += shad;
  if (error) return 2;
  s->last_time = t;
  s->initialized = 1;
  return 0;
}

int oracle_sensor_process(osensor *s, const ointerval *ivs, int count, oevent *out, size_t cap,
                          size_t *n_out, int nthreads) {
  /* upload_intervals (event_sensor.cu:274-289) */
  *n_out = 0;
  if (!s->initialized || count <= 0) return 3;
  double previous = s->last_time, cells = 0;
  for (int k = 0; k < count; ++k) {
    const ointerval *iv = &ivs[k];
    if (!isfinite(iv->t0) || !isfinite(iv->t1) || iv->t0 != previous || iv->t1 <= iv->t0) return 3;
    cells += (iv->t1 - iv->t0) / s->photo.integration_step;
    previous = iv->t1;
  }
  if (cells > 1000000) return 3;
  const int n = s->scene.width * s->scene.height, width = s->scene.width;
  const int maxev = s->max_events;
  double *ev_t = (double *)malloc(sizeof(double) * (size_t)n * maxev);
  int32_t *ev_p = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * maxev);
  float *ev_d = (float *)malloc(sizeof(float) * (size_t)n * maxev);
  int *ev_n = (int *)calloc((size_t)n, sizeof(int));
  int err_capacity = 0, err_optical = 0;
  const int nt = thread_count(nthreads);
  (void)nt;
  uint64_t prim = 0, shad = 0;
  /* generate_pixels (event_sensor.cu:29-60) */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt) reduction(+ : prim, shad)
  for (int i = 0; i < n; ++i) {
    double *lt = ev_t + (size_t)i * maxev;
    int32_t *lp = ev_p + (size_t)i * maxev;
    int cnt = 0, failed = 0;
    uint64_t a = 0, b = 0;
    opixel_state st = s->states[i];
    uint8_t *mark = s->classify ? &s->margin[i] : NULL;
    for (int k = 0; k < count && !failed; ++k) {
      const ointerval *iv = &ivs[k];
      int steps = (int)ceil((iv->t1 - iv->t0) / s->photo.integration_step);
      double dt = (iv->t1 - iv->t0) / steps;
      for (int step = 0; step < steps; ++step) {
        double t0 = iv->t0 + step * dt, t1 = step + 1 == steps ? iv->t1 : iv->t0 + (step + 1) * dt;
        ostate pose;
        oracle_optical_state_at(iv, (t0 + t1) * .5, &pose);
        double rad;
        float depth;
        int valid;
        sample_pixel_m(&s->scene, i, &pose, &rad, &depth, &valid, &a, &b, mark);
        if (!valid || !isfinite(rad)) { failed = 2; break; }
        double rate = rad * s->photo.electrons_per_radiance + s->photo.dark_electrons;
        int emitted = advance_pixel(&st, &s->params, rate, t0, t1, lt + cnt, lp + cnt, maxev - cnt);
        if (emitted < 0) { failed = 1; break; }
        if (mark) {
          /* the two shadow circuits see the same light */
          seq_push(&s->seq[3 * (size_t)i], lp + cnt, emitted);
          for (int v = 0; v < 2; ++v) {
            double vt[64];
            int32_t vp[64];
            const int e = advance_pixel(&s->shifted[2 * (size_t)i + v], &s->params, rate, t0, t1, vt, vp, 64);
            if (e < 0) *mark |= 2;
            else seq_push(&s->seq[3 * (size_t)i + 1 + v], vp, e);
          }
        }
        cnt += emitted;
      }
    }
    s->states[i] = st;
    if (!failed) {
      int interval = 0;
      for (int j = 0; j < cnt; ++j) {
        while (interval + 1 < count && lt[j] > ivs[interval].t1) ++interval;
        ostate pose;
        oracle_optical_state_at(&ivs[interval], lt[j], &pose);
        double rad;
        float depth;
        int valid;
        uint8_t depth_mark = 0;
        sample_pixel_m(&s->scene, i, &pose, &rad, &depth, &valid, &a, &b, mark ? &depth_mark : NULL);
        if (!valid) { failed = 2; break; }
        if (depth_mark) *mark |= 4;
        ev_d[(size_t)i * maxev + j] = depth;
      }
    }
    prim += a;
    shad += b;
    if (failed == 1) {
#pragma omp atomic write
      err_capacity = 1;
    } else if (failed == 2) {
#pragma omp atomic write
      err_optical = 1;
    } else
      ev_n[i] = cnt;
  }
  s->primary_rays += prim;
  s->shadow_rays += shad;
  int status = 0;
  if (err_capacity) status = 1;
  else if (err_optical) status = 2;
  if (!status) {
    size_t total = 0;
    for (int i = 0; i < n; ++i) total += ev_n[i];
    oevent *gen = (oevent *)malloc(sizeof(oevent) * (total ? total : 1));
    size_t k = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < ev_n[i]; ++j) {
        oevent e;
        e.timestamp = ev_t[(size_t)i * maxev + j];
        e.x = (int16_t)(i % width);
        e.y = (int16_t)(i / width);
        e.polarity = (int8_t)ev_p[(size_t)i * maxev + j];
        e.depth = ev_d[(size_t)i * maxev + j];
        gen[k++] = e;
      }
    /* collect_events (event_sensor.cu:296-305) */
    status = oracle_readout_submit(s->readout, gen, total, ivs[count - 1].t1, out, cap, n_out);
    s->last_time = ivs[count - 1].t1;
    free(gen);
  }
  free(ev_t); free(ev_p); free(ev_d); free(ev_n);
  return status;
}

int oracle_sensor_drain(osensor *s, oevent *out, size_t cap, size_t *n_out) {
  return oracle_readout_drain(s->readout, out, cap, n_out);
}
void oracle_sensor_states(const osensor *s, opixel_state *out) {
  memcpy(out, s->states, sizeof(opixel_state) * (size_t)s->scene.width * s->scene.height);
}
size_t oracle_sensor_dropped(const osensor *s) { return s->readout->dropped; }
uint64_t oracle_sensor_rays(const osensor *s, int shadow) { return shadow ? s->shadow_rays : s->primary_rays; }
