// Camera / light trajectory: src/trajectory.cpp semantics in FP32.
#include "app_trajectory.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace dvs_app {
namespace {

float clampf(float x, float lo, float hi) { return std::max(lo, std::min(x, hi)); }

// Auto-clamped (monotone cubic) key slopes (trajectory.cpp:26-81): the
// weighted harmonic mean of the neighbouring secant slopes, zero at extrema.
std::vector<float> key_slopes(const std::vector<float> &t, const std::vector<float> &y) {
  const size_t n = t.size();
  std::vector<float> m(n, 0.0f);
  if (n <= 1) return m;
  if (n == 2) {
    const float h = t[1] - t[0];
    const float d = std::fabs(h) > 1e-12f ? (y[1] - y[0]) / h : 0.0f;
    m[0] = m[1] = d;
    return m;
  }
  std::vector<float> h(n - 1), d(n - 1);
  for (size_t i = 0; i + 1 < n; ++i) {
    h[i] = t[i + 1] - t[i];
    d[i] = std::fabs(h[i]) > 1e-12f ? (y[i + 1] - y[i]) / h[i] : 0.0f;
  }
  m[0] = d[0];
  m[n - 1] = d[n - 2];
  for (size_t i = 1; i + 1 < n; ++i) {
    const float d0 = d[i - 1], d1 = d[i];
    if (d0 == 0.0f || d1 == 0.0f || d0 * d1 <= 0.0f) continue;
    const float w1 = 2.0f * h[i] + h[i - 1], w2 = h[i] + 2.0f * h[i - 1];
    const float denom = w1 / d0 + w2 / d1;
    m[i] = std::fabs(denom) > 1e-12f ? (w1 + w2) / denom : 0.0f;
  }
  return m;
}

Quat rotvec_exp(V3 r) {
  const float theta = norm(r);
  if (theta < 1e-8f) return qnormalized(Quat(1.0f, 0.5f * r.x, 0.5f * r.y, 0.5f * r.z));
  const V3 axis = r / theta;
  const float half = 0.5f * theta, s = std::sin(half);
  return qnormalized(Quat(std::cos(half), s * axis.x, s * axis.y, s * axis.z));
}

V3 quat_log(const Quat &q_in) {
  Quat q = qnormalized(q_in);
  if (q.w < 0.0f) q = qneg(q);  // short arc
  const V3 v(q.x, q.y, q.z);
  const float s = norm(v);
  if (s < 1e-8f) return 2.0f * v;
  const float theta = 2.0f * std::atan2(s, q.w);
  return v * (theta / s);
}

V3 unit_vector_rate(V3 v, V3 vdot) {
  const float n = norm(v);
  if (n < 1e-12f) return V3();
  const float k = dot(v, vdot);
  return vdot / n - v * (k / (n * n * n));
}

}  // namespace

dvs_optical_state to_optical_state(const TrajectoryState &s) {
  dvs_optical_state p{};
  p.position = dvs_float3{s.position.x, s.position.y, s.position.z};
  p.velocity = dvs_float3{s.linear_velocity.x, s.linear_velocity.y, s.linear_velocity.z};
  p.light = dvs_float3{s.light_direction.x, s.light_direction.y, s.light_direction.z};
  p.light_rate = dvs_float3{s.light_direction_rate.x, s.light_direction_rate.y, s.light_direction_rate.z};
  p.rotation.x = s.quaternion.x;
  p.rotation.y = s.quaternion.y;
  p.rotation.z = s.quaternion.z;
  p.rotation.w = s.quaternion.w;
  p.intensity = s.light_intensity;
  p.intensity_rate = s.light_intensity_rate;
  return p;
}

// ---- BezierChannel ------------------------------------------------------------
void BezierChannel::build(const std::vector<float> &times, const std::vector<float> &values) {
  keys_.clear();
  if (times.size() != values.size()) throw std::invalid_argument("ScalarBezierCurve::build_auto_clamped: size mismatch");
  const size_t n = times.size();
  if (n == 0) return;
  for (size_t i = 1; i < n; ++i)
    if (!(times[i] > times[i - 1]))
      throw std::invalid_argument("ScalarBezierCurve::build_auto_clamped: timestamps must be strictly increasing");
  keys_.resize(n);
  for (size_t i = 0; i < n; ++i) {
    Key &k = keys_[i];
    k.t = k.lt = k.rt = times[i];
    k.v = k.lv = k.rv = values[i];
  }
  if (n == 1) return;
  const std::vector<float> m = key_slopes(times, values);
  // handles a third of the way into each segment along the key slope
  for (size_t i = 0; i + 1 < n; ++i) {
    const float t0 = times[i], t1 = times[i + 1], h = t1 - t0;
    keys_[i].rt = t0 + h / 3.0f;
    keys_[i].rv = values[i] + m[i] * h / 3.0f;
    keys_[i + 1].lt = t1 - h / 3.0f;
    keys_[i + 1].lv = values[i + 1] - m[i + 1] * h / 3.0f;
  }
}

int BezierChannel::segment(float t) const {
  const int n = int(keys_.size());
  if (n < 2) return -1;
  if (t <= keys_.front().t) return 0;
  if (t >= keys_.back().t) return n - 2;
  const auto it = std::upper_bound(keys_.begin(), keys_.end(), t, [](float x, const Key &k) { return x < k.t; });
  return std::max(0, std::min(int(it - keys_.begin()) - 1, n - 2));
}

// de Casteljau in difference form: a constant curve stays exactly constant.
float BezierChannel::curve(float p0, float p1, float p2, float p3, float u) {
  const float a = p0 + u * (p1 - p0), b = p1 + u * (p2 - p1), c = p2 + u * (p3 - p2);
  const float d = a + u * (b - a), e = b + u * (c - b);
  return d + u * (e - d);
}

float BezierChannel::slope(float p0, float p1, float p2, float p3, float u) {
  const float v = 1.0f - u;
  return 3.0f * v * v * (p1 - p0) + 6.0f * v * u * (p2 - p1) + 3.0f * u * u * (p3 - p2);
}

// Curve parameter u with x(u) = t: Newton from the linear guess (8 steps,
// stop when a step is below 1e-7), then 24 bisections if Newton did not settle.
float BezierChannel::parameter_at(const Key &a, const Key &b, float t) {
  const float x0 = a.t, x1 = a.rt, x2 = b.lt, x3 = b.t;
  const float span = x3 - x0;
  if (span <= 1e-12f) return 0.0f;
  float u = clampf((t - x0) / span, 0.0f, 1.0f);
  for (int i = 0; i < 8; ++i) {
    const float x = curve(x0, x1, x2, x3, u), dx = slope(x0, x1, x2, x3, u);
    if (std::fabs(dx) < 1e-10f) break;
    const float next = clampf(u - (x - t) / dx, 0.0f, 1.0f);
    if (std::fabs(next - u) < 1e-7f) return next;
    u = next;
  }
  float lo = 0.0f, hi = 1.0f;
  for (int i = 0; i < 24; ++i) {
    const float mid = 0.5f * (lo + hi);
    if (curve(x0, x1, x2, x3, mid) < t) lo = mid;
    else hi = mid;
  }
  return 0.5f * (lo + hi);
}

float BezierChannel::evaluate(float t) const {
  if (keys_.empty()) return 0.0f;
  if (keys_.size() == 1 || t <= keys_.front().t) return keys_.front().v;
  if (t >= keys_.back().t) return keys_.back().v;
  const int s = segment(t);
  const Key &a = keys_[size_t(s)], &b = keys_[size_t(s) + 1];
  return curve(a.v, a.rv, b.lv, b.v, parameter_at(a, b, t));
}

float BezierChannel::derivative(float t) const {
  if (keys_.size() < 2) return 0.0f;
  // the segment comes from the query clamped just inside the key range; the
  // curve parameter from the query itself (trajectory.cpp:283-311)
  const float eps = 1e-7f;
  float tc = t;
  if (tc < keys_.front().t + eps) tc = keys_.front().t + eps;
  if (tc > keys_.back().t - eps) tc = keys_.back().t - eps;
  const int s = segment(tc);
  const Key &a = keys_[size_t(s)], &b = keys_[size_t(s) + 1];
  const float u = parameter_at(a, b, t);
  const float dx = slope(a.t, a.rt, b.lt, b.t, u), dy = slope(a.v, a.rv, b.lv, b.v, u);
  if (std::fabs(dx) < 1e-12f) return 0.0f;
  return dy / dx;
}

// ---- CameraTrajectory -----------------------------------------------------------
CameraTrajectory::CameraTrajectory(const std::vector<FrameData> &frames, const SceneConfig &scene) {
  const float fps = scene.fps;
  if (!std::isfinite(fps) || fps <= 0 || scene.translation.size() != 3 || scene.rotation.size() != 3)
    throw std::invalid_argument("trajectory requires positive fps and three-component mount transforms");
  const V3 mount_t(scene.translation[0], scene.translation[1], scene.translation[2]);
  // mount rotation from Euler angles, Z * Y * X
  const M3 mount_r = axis_angle(scene.rotation[2], V3(0, 0, 1)) * axis_angle(scene.rotation[1], V3(0, 1, 0)) *
                     axis_angle(scene.rotation[0], V3(1, 0, 0));
  if (frames.empty()) return;
  const size_t n = frames.size();
  std::vector<float> times(n), xs(n), ys(n), zs(n), lxs(n), lys(n), lzs(n), intensities(n);
  bool increasing = true;
  for (size_t i = 0; i < n; ++i) {
    times[i] = float(frame_time(frames[i], fps));
    if (!std::isfinite(times[i])) throw std::invalid_argument("non-finite trajectory timestamp");
    if (i > 0 && !(times[i] > times[i - 1])) increasing = false;
  }
  if (!increasing) throw std::invalid_argument("trajectory timestamps must be strictly increasing");

  rotations_.resize(n);
  M3 identity;
  for (size_t i = 0; i < n; ++i) {
    const FrameData &f = frames[i];
    M3 gram = transpose(f.camera_world) * f.camera_world;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) gram.m[a][b] -= identity.m[a][b];
    if (!all_finite(f.camera_origin) || !all_finite(f.camera_world) || !all_finite(f.light_dir) ||
        norm(f.light_dir) < 1e-12f || !std::isfinite(f.light_intensity) || f.light_intensity < 0 ||
        frobenius(gram) > 2e-3f || determinant(f.camera_world) <= 0)
      throw std::invalid_argument("trajectory requires finite rigid poses and valid world lighting");
    const V3 centre = f.camera_origin + f.camera_world * mount_t;
    xs[i] = centre.x;
    ys[i] = centre.y;
    zs[i] = centre.z;
    Quat q = qnormalized(quat_from_matrix(f.camera_world * mount_r));
    if (i > 0 && qdot(q, rotations_[i - 1]) < 0.0f) q = qneg(q);  // sign continuity
    rotations_[i] = qnormalized(q);
    V3 ld = f.light_dir;
    const float ln = norm(ld);
    ld = ln > 1e-12f ? ld / ln : V3(0, 0, 1);
    lxs[i] = ld.x;
    lys[i] = ld.y;
    lzs[i] = ld.z;
    intensities[i] = f.light_intensity;
  }
  px_.build(times, xs);
  py_.build(times, ys);
  pz_.build(times, zs);
  // orientation keys: normalized, sign-continuous; phase i at key i
  for (size_t i = 0; i < n; ++i) {
    rotations_[i] = qnormalized(rotations_[i]);
    if (i > 0 && qdot(rotations_[i], rotations_[i - 1]) < 0.0f) rotations_[i] = qneg(rotations_[i]);
  }
  std::vector<float> phase(n);
  for (size_t i = 0; i < n; ++i) phase[i] = float(i);
  phase_.build(times, phase);
  lx_.build(times, lxs);
  ly_.build(times, lys);
  lz_.build(times, lzs);
  intensity_.build(times, intensities);
}

bool CameraTrajectory::valid() const {
  return px_.valid() && py_.valid() && pz_.valid() && phase_.valid() && !rotations_.empty();
}

void CameraTrajectory::rotation_at(float t, Quat *q_out, M3 *R_out, V3 *omega_out) const {
  *q_out = Quat();
  *R_out = M3();
  *omega_out = V3();
  const int n = int(rotations_.size());
  const float phase = phase_.evaluate(t), phase_rate = phase_.derivative(t);
  if (n < 2) return;
  const int seg = std::max(0, std::min(int(std::floor(phase)), n - 2));
  const float alpha = clampf(phase - float(seg), 0.0f, 1.0f);
  const Quat &q0 = rotations_[size_t(seg)], &q1 = rotations_[size_t(seg) + 1];
  Quat rel = qnormalized(qmul(qconj(q0), q1));
  if (rel.w < 0.0f) rel = qneg(rel);
  const V3 rho = quat_log(rel);
  const Quat q = qnormalized(qmul(q0, rotvec_exp(alpha * rho)));
  const M3 R = qmatrix(q);
  *q_out = q;
  *R_out = R;
  *omega_out = R * (phase_rate * rho);  // body rate alpha' * rho, in the world frame
}

TrajectoryState CameraTrajectory::evaluate(float t) const {
  TrajectoryState out;
  out.timestamp = t;
  if (!valid()) return out;
  const float tc = clampf(t, start_time(), end_time());
  out.timestamp = tc;
  out.position = V3(px_.evaluate(tc), py_.evaluate(tc), pz_.evaluate(tc));
  out.linear_velocity = V3(px_.derivative(tc), py_.derivative(tc), pz_.derivative(tc));
  rotation_at(tc, &out.quaternion, &out.orientation, &out.angular_velocity);
  const V3 raw(lx_.evaluate(tc), ly_.evaluate(tc), lz_.evaluate(tc));
  const V3 raw_rate(lx_.derivative(tc), ly_.derivative(tc), lz_.derivative(tc));
  const float ln = norm(raw);
  if (ln > 1e-12f) {
    out.light_direction = raw / ln;
    out.light_direction_rate = unit_vector_rate(raw, raw_rate);
  } else {
    out.light_direction = V3(0, 0, 1);
    out.light_direction_rate = V3();
  }
  out.light_intensity = intensity_.evaluate(tc);
  out.light_intensity_rate = intensity_.derivative(tc);
  return out;
}

}  // namespace dvs_app
