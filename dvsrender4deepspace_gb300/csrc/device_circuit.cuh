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
  // false once refractory_until <= the start of a cell: the deadline then
  // stays in the past for every later cell until an event sets a new one
  bool refractory;
};

// The FP32 forms of the parameters the no-event path reads, converted once per
// chunk instead of per cell.
struct PixelParamsF {
  float charge, leak;
  bool reset_noise;
};
__device__ __forceinline__ PixelParamsF pixel_params_f32(const PixelParams &p) {
  return PixelParamsF{(float)p.charge_scale, (float)p.reference_leak, p.reset_noise_std > 0};
}

// The FP64 parts of advance_pixel_f32 are separate, non-inlined functions:
// inlined, the compiler hoisted parts of them (promotions of the FP32 state,
// FP64 compares) into the no-event path, where they ran on every cell --
// 30-44 FP64 instructions per warp and cell, on a GPU whose FP64 rate is a
// small fraction of its FP32 rate.  Called only where the arithmetic needs
// them (an event, a refractory reset, a nonzero leak); same operations, same
// results.
template <class Rng>
__device__ __noinline__ float reset_noise_draw(double stddev, Rng &rng) {
  return (float)(stddev * curand_normal_double(&rng));
}
// The leak extremum (FP64): the time at which the leaking reference stops
// approaching the receptor, as a new segment end if it comes first.
__device__ __noinline__ float leak_segment_end(const PixelParams &p, float rate, float u, float boundary) {
  const double rate_d = rate, x = exp((double)u), target = rate_d + p.charge_scale * p.reference_leak;
  if (x > target && target > rate_d) {
    double extremum;
    if (rate_d > 0) extremum = -p.charge_scale / rate_d * log((1.0 / target - 1.0 / rate_d) / (1.0 / x - 1.0 / rate_d));
    else extremum = p.charge_scale * (1.0 / target - 1.0 / x);
    if (extremum > 1e-15 && extremum < (double)boundary) return (float)extremum;
  }
  return boundary;
}
// The crossing time in FP64 from the FP32 state, as an offset into the segment,
// and the receptor log at that time (FP32).
struct Crossing {
  double hi;
  float u;
};
__device__ __noinline__ Crossing crossing_f64(const PixelParams &p, float rate, float u, float ref, float level,
                                              float boundary, bool immediate, int polarity) {
  const double rate_d = rate, ud = u, refd = ref, leveld = level, bnd = boundary;
  double lo = 0, hi = bnd;
  if (immediate) hi = 0;
  else if (p.reference_leak == 0) {
    const double target_inverse = exp(-(refd + leveld)), initial_inverse = exp(-ud);
    if (rate_d > 0) {
      const double stationary_inverse = 1.0 / rate_d;
      hi = -p.charge_scale / rate_d * log1p((target_inverse - initial_inverse) / (initial_inverse - stationary_inverse));
    } else hi = p.charge_scale * (target_inverse - initial_inverse);
    hi = fmin(bnd, fmax(0.0, hi));
  } else
    for (int j = 0; j < 48; ++j) {
      const double mid = (lo + hi) * .5;
      const double cm = receptor_log_at(ud, rate_d, mid, p.charge_scale) - refd + p.reference_leak * mid;
      if (polarity ? cm >= leveld : cm <= leveld) hi = mid; else lo = mid;
    }
  return Crossing{hi, (float)receptor_log_at(ud, rate_d, hi, p.charge_scale)};
}

// Time inside the cell is an FP32 offset from the cell start (t0) and the
// refractory deadline an FP32 offset too, formed from the FP64 deadline only
// while the pixel is still refractory, so the no-event path has no FP64
// arithmetic (GB300's FP64 pipe is narrow, and one lane that uses it costs
// its warp the whole instruction); absolute event times and deadlines are
// formed in FP64 only when an event happens.
template <class Rng>
__device__ int advance_pixel_f32(PixelRegsF &s, const PixelParams &p, const PixelParamsF &pf, float rate, double t0,
                                 float dt, double *out_t, int8_t *out_p, int capacity, Rng &rng) {
  if (!(dt > 0)) return 0;
  const float charge = pf.charge, leak = pf.leak;
  int count = 0;
  // a deadline in the past gives ref_off <= 0, which no offset in the cell is below
  float off = 0.0f, ref_off = -1.0f;
  if (s.refractory) {
    ref_off = (float)(s.refractory_until - t0);
    s.refractory = ref_off > 0.0f;
  }
  float u = s.receptor_log;
  int passes = 0;
  // With a constant rate the receptor moves monotonically toward it, so once
  // it has reached the leak target (the extremum) it stays past it for the
  // rest of the cell: there is at most one extremum split per cell.  The
  // FP32 state at the split can round to a hair before the target, and
  // recomputing the extremum from it would give ever shorter splits that an
  // FP32 offset cannot even add; so after one split it is not looked for again.
  bool past_extremum = false;
  while (off < dt) {
    if (++passes > 4096) return -2;  // bounded: see kErrStalled
    if (off < ref_off) {
      const float end = fminf(dt, ref_off);
      u = receptor_log_at_f(u, rate, end - off, charge);
      off = end;
      s.reference_log = u;
      if (off < dt || off == ref_off) {
        if (off >= ref_off && s.reset_pending) {
          if (pf.reset_noise) s.reference_log += reset_noise_draw(p.reset_noise_std, rng);
          s.reset_pending = false;
        }
      }
      if (off >= dt) break;
    } else if (s.reset_pending) {
      if (pf.reset_noise) s.reference_log += reset_noise_draw(p.reset_noise_std, rng);
      s.reset_pending = false;
    }
    const float remaining = dt - off;
    float boundary = remaining;
    if (leak > 0 && !past_extremum) boundary = leak_segment_end(p, rate, u, boundary);  // FP64: places the end
    const float c0 = u - s.reference_log;
    const float ub = receptor_log_at_f(u, rate, boundary, charge);
    const float cb = ub - s.reference_log + leak * boundary;
    int polarity = -1;
    float level = 0;
    if (c0 >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (c0 <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    else if (cb >= s.threshold_pos) { polarity = 1; level = s.threshold_pos; }
    else if (cb <= -s.threshold_neg) { polarity = 0; level = -s.threshold_neg; }
    if (polarity < 0) {
      u = ub;
      s.reference_log -= leak * boundary;
      if (boundary == remaining) off = dt;
      else { off += boundary; past_extremum = true; }
      continue;
    }
    if (count == capacity) return -1;
    const Crossing x = crossing_f64(p, rate, u, s.reference_log, level, boundary,
                                    c0 >= s.threshold_pos || c0 <= -s.threshold_neg, polarity);
    const double hi = x.hi;
    u = x.u;
    const double t_event = t0 + (double)off + hi;
    off = fminf(dt, off + (float)hi);
    out_t[count] = t_event;
    out_p[count] = (int8_t)polarity;
    ++count;
    s.reference_log = u;
    s.refractory_until = t_event + p.refractory_time;
    ref_off = (float)(s.refractory_until - t0);
    s.refractory = true;
    s.reset_pending = true;
  }
  s.receptor_log = u;
  return count;
}

// log of the Poisson pmf, k log(mu) - mu - log(k!), in FP32 without the
// cancellation of large terms that the direct form suffers at large means.
// Below k = 10 the direct form with lgammaf (the terms are small there).
// From k = 10, Stirling's series log k! = (k + 1/2) log k - k + log(2 pi)/2
// + 1/(12k) - 1/(360k^3) + 1/(1260k^5) (truncation error below 1e-10) turns
// k log(mu) - mu - (k log k - k) into -mu h(x), x = (k - mu)/mu and
// h(x) = (1 + x) log1p(x) - x, which is summed as its power series
// sum_{n>=2} (-1)^n x^n / (n (n - 1)) for |x| < 1/4, where the closed form
// would cancel.  Against FP64 lgamma the absolute error stays below 1e-5
// wherever the pmf is above e^-25, for means from 10 to 1e6.
__device__ __forceinline__ float poisson_log_pmf(float k, float mu) {
  if (k < 10.0f) return k * logf(mu) - mu - lgammaf(k + 1.0f);
  const float x = (k - mu) / mu;
  float h;
  if (fabsf(x) < 0.25f) {
    float acc = 1.0f / 132.0f;  // n = 12
    acc = fmaf(acc, x, -1.0f / 110.0f);
    acc = fmaf(acc, x, 1.0f / 90.0f);
    acc = fmaf(acc, x, -1.0f / 72.0f);
    acc = fmaf(acc, x, 1.0f / 56.0f);
    acc = fmaf(acc, x, -1.0f / 42.0f);
    acc = fmaf(acc, x, 1.0f / 30.0f);
    acc = fmaf(acc, x, -1.0f / 20.0f);
    acc = fmaf(acc, x, 1.0f / 12.0f);
    acc = fmaf(acc, x, -1.0f / 6.0f);
    acc = fmaf(acc, x, 0.5f);  // n = 2
    h = acc * x * x;
  } else {
    h = (1.0f + x) * log1pf(x) - x;
  }
  const float ik = 1.0f / k, ik2 = ik * ik;
  const float series = ik * (1.0f / 12.0f - ik2 * (1.0f / 360.0f - ik2 * (1.0f / 1260.0f)));
  const float half_log_2pi = 0.918938533f;  // log(2 pi) / 2
  return -mu * h - 0.5f * logf(k) - half_log_2pi - series;
}

// A uniform draw in (0, 1] from the top 23 bits of one 32-bit Philox output:
// the bits are the mantissa of a float in [1, 2), and 2 minus it lies in
// [2^-23, 1].  Integer and FP32 operations only -- no integer-to-float
// conversion instruction -- with the resolution of an FP32 uniform near 1.
__device__ __forceinline__ float philox_uniform(curandStatePhilox4_32_10_t &st) {
  return 2.0f - __uint_as_float(0x3f800000u | (curand(&st) >> 9));
}
// floor(x) for |x| < 2^23 by one addition rounded toward -inf: at 2^23 the
// float spacing is 1, so x + 2^23 rounds down to the integer below it
// (exact for every float in that range, negative ones included).
__device__ __forceinline__ float floor_small(float x) {
  return __fadd_rd(x, 8388608.0f) - 8388608.0f;
}

// Poisson draw for means of 10 and more by the transformed rejection method
// with squeeze of W. Hormann, "The transformed rejection method for
// generating Poisson random variables", Insurance: Mathematics and Economics
// 12 (1993) 39-45 (algorithm PTRS).  A candidate k comes from a transformed
// uniform U, a second uniform V accepts it at once inside the squeeze (about
// 90 % of candidates at these means), and the rest are decided by the exact
// test log(V * alpha / (a / us^2 + b)) <= log pmf(k), all in FP32 (the pmf
// through poisson_log_pmf).  With one lane in ten taking the test nearly
// every warp runs it, so it must not run on the GPU's narrow FP64 pipe.  The
// constants are the paper's.  Every candidate takes two uniforms; after 64
// rejected candidates (a probability far below 1e-60) the draw falls back to
// the rounded normal.  Candidates are clamped to |k| < 2^23 before the
// floor: means stop at 1e6, so a clamped candidate is rejected either way.
__device__ __forceinline__ float poisson_ptrs(curandStatePhilox4_32_10_t &st, float mu) {
  const float smu = sqrtf(mu);
  const float b = 0.931f + 2.53f * smu;
  const float a = -0.059f + 0.02483f * b;
  const float inv_alpha = 1.1239f + 1.1328f / (b - 3.4f);
  const float v_r = 0.9277f - 3.6224f / (b - 2.0f);
  for (int attempt = 0; attempt < 64; ++attempt) {
    const float U = philox_uniform(st) - 0.5f;  // (-1/2, 1/2]
    const float V = philox_uniform(st);         // (0, 1]
    const float us = 0.5f - fabsf(U);
    if (us < 0.013f && V > us) continue;  // outside the hat's usable part (also guards us == 0)
    const float x = (2.0f * a / us + b) * U + mu + 0.43f;
    const float k = floor_small(fminf(fmaxf(x, -8388607.0f), 8388607.0f));
    if (us >= 0.07f && V <= v_r) return k;
    if (k < 0.0f) continue;
    const float lhs = logf(V) + logf(inv_alpha) - logf(a / (us * us) + b);
    if (lhs <= poisson_log_pmf(k, mu)) return k;
  }
  return fmaxf(0.0f, floorf(mu + smu * curand_normal(&st) + 0.5f));
}

// Photon count of one cell from a counter-based Philox stream (precision
// mode): inversion of the Poisson CDF by sequential search below a mean of 10
// (the photon-starved regime of the sensor), PTRS from 10 to 1e6, and above
// 1e6 the rounded normal approximation the reference's poisson_electrons
// uses there (include/dvs/photon_noise.cuh:7).  The stream is keyed by
// (seed, pixel) and placed at the cell's absolute index, so the draws do not
// depend on how cells are batched.
__device__ __forceinline__ float poisson_electrons_philox(curandStatePhilox4_32_10_t &st, float lambda) {
  if (!(lambda > 0)) return 0;
  if (lambda > 1e6f) return fmaxf(0.0f, floorf(lambda + sqrtf(lambda) * curand_normal(&st) + 0.5f));
  if (lambda >= 10.0f) return poisson_ptrs(st, lambda);
  const float u = philox_uniform(st);  // (0, 1]
  float p = expf(-lambda), F = p;
  float k = 0.0f;  // counted in float: no conversion per step
  while (u > F && k < 512.0f) {
    k += 1.0f;
    p *= lambda / k;
    const float next = F + p;
    if (!(next > F)) break;  // the CDF stopped growing in float (tail mass below its last ulp)
    F = next;
  }
  return k;
}
// The pixel's Philox stream at a place fixed by the cell's start time: a
// 64-bit mix (the SplitMix64 finalizer) of the bits of t0, aligned to 16
// draws, so distinct cells get disjoint draws whatever their length and
// however they are batched.  Offsets 0..15 belong to the initialization.
__device__ __forceinline__ curandStatePhilox4_32_10_t philox_at(unsigned seed, int pixel, double cell_t0) {
  unsigned long long z = (unsigned long long)__double_as_longlong(cell_t0) + 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  curandStatePhilox4_32_10_t st;
  curand_init(seed, (unsigned long long)pixel, (z | 16ull) & ~15ull, &st);
  return st;
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
