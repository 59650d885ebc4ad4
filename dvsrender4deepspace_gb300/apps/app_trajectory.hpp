// Continuous camera and light trajectory of the drop-in apps
// (include/dvs/trajectory.hpp, src/trajectory.cpp:26-81,114-331,406-568,609-790),
// in FP32 like the reference: every channel is a Blender-style cubic Bezier
// F-curve with auto-clamped handles (monotone-cubic slopes), evaluated by
// solving x(u) = t; orientation follows a phase curve and is interpolated on
// SO(3) as q0 * exp(alpha * log(q0^-1 q1)).  Velocities and rates are the
// analytic derivatives of those curves.
#pragma once
#include <vector>

#include "app_config.hpp"
#include "app_math.hpp"
#include "app_scene.hpp"
#include "dvs_gb300.h"

namespace dvs_app {

struct TrajectoryState {
  float timestamp = 0.0f;
  V3 position;
  M3 orientation;
  Quat quaternion;
  V3 linear_velocity, angular_velocity;
  V3 light_direction = V3(0, 0, 1), light_direction_rate;
  float light_intensity = 0.0f, light_intensity_rate = 0.0f;
};

// OpticalState of a trajectory sample (include/dvs/raycast.hpp:17-22).
dvs_optical_state to_optical_state(const TrajectoryState &s);

class BezierChannel {
 public:
  // Keys at strictly increasing times; throws std::invalid_argument otherwise.
  void build(const std::vector<float> &times, const std::vector<float> &values);
  bool valid() const { return !keys_.empty(); }
  float start_time() const { return keys_.empty() ? 0.0f : keys_.front().t; }
  float end_time() const { return keys_.empty() ? 0.0f : keys_.back().t; }
  float evaluate(float t) const;
  float derivative(float t) const;

 private:
  struct Key {
    float t = 0, v = 0;          // the key
    float lt = 0, lv = 0;        // left handle
    float rt = 0, rv = 0;        // right handle
  };
  int segment(float t) const;
  static float curve(float p0, float p1, float p2, float p3, float u);
  static float slope(float p0, float p1, float p2, float p3, float u);
  static float parameter_at(const Key &a, const Key &b, float t);
  std::vector<Key> keys_;
};

class CameraTrajectory {
 public:
  CameraTrajectory(const std::vector<FrameData> &frames, const SceneConfig &scene);
  bool valid() const;
  float start_time() const { return px_.start_time(); }
  float end_time() const { return px_.end_time(); }
  TrajectoryState evaluate(float t) const;

 private:
  void rotation_at(float t, Quat *q, M3 *R, V3 *omega) const;
  BezierChannel px_, py_, pz_, lx_, ly_, lz_, intensity_, phase_;
  std::vector<Quat> rotations_;
};

}  // namespace dvs_app
