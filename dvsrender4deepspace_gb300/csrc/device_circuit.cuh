// Device-side pixel circuit of the GB300 DVS path (include/dvs/pixel_model.hpp
// semantics, FP64) and the cuRAND photon-count draw.  Internal linkage.
#pragma once
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "kernels.h"

namespace dvsgb {
namespace {
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
    if (p.reference_leak > 0) {  // the leak extremum exists only with a leak: no exp(u) otherwise
      const double x = exp(u), target = rate + p.charge_scale * p.reference_leak;
      if (x > target && target > rate) {
        double extremum;
        if (rate > 0) extremum = -p.charge_scale / rate * log((1.0 / target - 1.0 / rate) / (1.0 / x - 1.0 / rate));
        else extremum = p.charge_scale * (1.0 / target - 1.0 / x);
        if (extremum > 1e-15 && extremum < boundary) boundary = extremum;
      }
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

// ---- FP32 circuit (precision mode) ------------------------------------------------
// The same pixel model with the receptor and contrast arithmetic in FP32 and
// everything that fixes when an event happens in FP64: absolute times,
// refractory deadlines, the leak extremum and the crossing-time root solve
// (done from the FP32 state promoted to FP64).  Events are the FP64 model's
// up to the FP32 rounding of the log voltages (~1e-6 of a 0.2 threshold).
__device__ __forceinline__ float receptor_log_at_f(float u, float rate, float dt, float charge) {
  if (dt <= 0) return u;
  rate = fmaxf(0.0f, rate);
  const float x = expf(u);
  if (rate == 0) return u - log1pf(x * dt / charge);
  const float a = expf(-rate * dt / charge), b = -expm1f(-rate * dt / charge);
  return -logf(a / x + b / rate);
}

struct PixelRegsF {
  float receptor_log, reference_log;
  double refractory_until;
  float threshold_pos, threshold_neg;
  bool reset_pending;
};

__device__ int advance_pixel_f32(PixelRegsF &s, const PixelParams &p, double rate_d, double t0, double t1,
                                 double *out_t, int8_t *out_p, int capacity, curandStateXORWOW_t &rng) {
  if (t1 <= t0) return 0;
  const float rate = (float)rate_d, charge = (float)p.charge_scale, leak = (float)p.reference_leak;
  int count = 0;
  double cursor = t0;
  float u = s.receptor_log;
  int passes = 0;
  while (cursor < t1) {
    if (++passes > 4096) return -2;  // bounded: see kErrStalled
    if (cursor < s.refractory_until) {
      const double end = fmin(t1, s.refractory_until);
      u = receptor_log_at_f(u, rate, (float)(end - cursor), charge);
      cursor = end;
      s.reference_log = u;
      if (cursor < t1 || cursor == s.refractory_until) {
        if (cursor >= s.refractory_until && s.reset_pending) {
          if (p.reset_noise_std > 0) s.reference_log += (float)(p.reset_noise_std * curand_normal_double(&rng));
          s.reset_pending = false;
        }
      }
      if (cursor >= t1) break;
    } else if (s.reset_pending) {
      if (p.reset_noise_std > 0) s.reference_log += (float)(p.reset_noise_std * curand_normal_double(&rng));
      s.reset_pending = false;
    }
    const double remaining = t1 - cursor;
    double boundary = remaining;
    if (leak > 0) {  // leak extremum in FP64 (it places the segment end)
      const double x = exp((double)u), target = rate_d + p.charge_scale * p.reference_leak;
      if (x > target && target > rate_d) {
        double extremum;
        if (rate_d > 0) extremum = -p.charge_scale / rate_d * log((1.0 / target - 1.0 / rate_d) / (1.0 / x - 1.0 / rate_d));
        else extremum = p.charge_scale * (1.0 / target - 1.0 / x);
        if (extremum > 1e-15 && extremum < boundary) boundary = extremum;
      }
    }
    const float c0 = u - s.reference_log;
    const float ub = receptor_log_at_f(u, rate, (float)boundary, charge);
    const float cb = ub - s.reference_log + leak * (float)boundary;
    int polarity = -1;
    float level = 0;
    if (c0 >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (c0 <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    else if (cb >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (cb <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    if (polarity < 0) {
      u = ub;
      s.reference_log -= leak * (float)boundary;
      cursor += boundary;
      continue;
    }
    if (count == capacity) return -1;
    // crossing time in FP64 from the FP32 state
    const double ud = u, refd = s.reference_log, leveld = level;
    double lo = 0, hi = boundary;
    if (c0 >= s.threshold_pos || c0 <= -s.threshold_neg) hi = 0;
    else if (p.reference_leak == 0) {
      const double target_inverse = exp(-(refd + leveld)), initial_inverse = exp(-ud);
      if (rate_d > 0) {
        const double stationary_inverse = 1.0 / rate_d;
        hi = -p.charge_scale / rate_d * log1p((target_inverse - initial_inverse) / (initial_inverse - stationary_inverse));
      } else hi = p.charge_scale * (target_inverse - initial_inverse);
      hi = fmin(boundary, fmax(0.0, hi));
    } else
      for (int j = 0; j < 48; ++j) {
        const double mid = (lo + hi) * .5;
        const double cm = receptor_log_at(ud, rate_d, mid, p.charge_scale) - refd + p.reference_leak * mid;
        if (polarity ? cm >= leveld : cm <= leveld) hi = mid; else lo = mid;
      }
    u = (float)receptor_log_at(ud, rate_d, hi, p.charge_scale);
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

}  // namespace
}  // namespace dvsgb
