// C++17 facade over the dvs_gb300 C-ABI with the reference's class names and
// call shapes, so that the reference's apps (apps/main_dvs.cpp,
// apps/main_cam.cpp) and tests keep their structure when they switch to the
// GB300 path.  Header-only; link against libdvs_gb300.so.
//
//   reference                                   here
//   DeviceScene(bundle, config, root)            dvs_gb300::DeviceScene(mesh arrays, camera, ss, hapke)
//     (include/dvs/device_scene.hpp:5-15)          -- builds the BVH itself; no BVHBuilder::build call
//   EventSensor / DvsRayCaster                   dvs_gb300::DvsRayCaster
//     initialize, advance, advance_many,           same names; events come back as std::vector<dvs_event>
//     drain, dropped_events, peak_queue            (include/dvs/raycast.hpp:23-62)
//   CamRayCaster::render_main                    dvs_gb300::CamRayCaster::render_main
//     (include/dvs/raycast.hpp:64-86)              (quaternion pose instead of an Eigen matrix)
//
// Failures throw what the reference throws: std::invalid_argument for bad
// inputs, std::runtime_error for device status and CUDA errors.
#pragma once
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "dvs_gb300.h"

namespace dvs_gb300 {

inline void check(int status) {
  if (status == DVS_OK) return;
  const std::string msg = dvs_last_error();
  if (status == DVS_ERR_INVALID) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

class DeviceScene {
 public:
  DeviceScene(const std::vector<float> &vertices, const std::vector<float> &normals,
              const std::vector<uint32_t> &indices, const dvs_camera &camera, int supersample,
              const dvs_hapke &hapke, const std::vector<float> *albedos = nullptr, int leaf_size = 0,
              int geometry = 0, int builder = 0) {
    if (vertices.size() % 3 || normals.size() != vertices.size() || indices.size() % 3 ||
        (albedos && albedos->size() * 3 != vertices.size()))
      throw std::invalid_argument("invalid indexed mesh/BVH/material dimensions");
    dvs_bvh_params params{};
    params.leaf_size = leaf_size;
    params.precision = geometry;  // DVS_BVH_HALF_BOUNDS | DVS_BVH_WATERTIGHT
    params.builder = builder;     // DVS_BVH_BUILD_SAH (default) or DVS_BVH_BUILD_MORTON
    dvs_scene *s = nullptr;
    check(dvs_scene_create(vertices.data(), normals.data(), indices.data(), albedos ? albedos->data() : nullptr,
                           vertices.size() / 3, indices.size() / 3, &camera, supersample, &hapke, &params, &s));
    scene_.reset(s);
    camera_ = camera;
  }
  dvs_scene *get() const { return scene_.get(); }
  const dvs_camera &camera() const { return camera_; }
  dvs_scene_info info() const {
    dvs_scene_info i{};
    check(dvs_scene_info_get(scene_.get(), &i));
    return i;
  }

 private:
  struct Deleter {
    void operator()(dvs_scene *s) const { dvs_scene_destroy(s); }
  };
  std::unique_ptr<dvs_scene, Deleter> scene_;
  dvs_camera camera_{};
};

class SensorBatch;

class DvsRayCaster {
 public:
  DvsRayCaster(std::shared_ptr<DeviceScene> scene, const dvs_physic &physic, const dvs_sensor_options *options = nullptr)
      : scene_(std::move(scene)) {
    dvs_sensor *s = nullptr;
    check(dvs_sensor_create(scene_->get(), &physic, options, &s));
    sensor_.reset(s);
  }
  void initialize(const dvs_optical_state &state, double timestamp) {
    check(dvs_sensor_initialize(sensor_.get(), &state, timestamp));
  }
  void advance(const dvs_optical_state &start, const dvs_optical_state &end, double t0, double t1,
               std::vector<dvs_event> &events) {
    dvs_optical_interval iv{start, end, t0, t1};
    advance_many(std::vector<dvs_optical_interval>{iv}, events);
  }
  void advance_many(const std::vector<dvs_optical_interval> &intervals, std::vector<dvs_event> &events) {
    size_t n = 0;
    check(dvs_sensor_process(sensor_.get(), intervals.data(), intervals.size(), &n));
    read(n, events);
  }
  // EventSensor::process_adaptive (include/dvs/raycast.hpp:40-43): false when
  // the convergence gate rejected the window (nothing changed; retry smaller).
  bool advance_adaptive(const std::vector<dvs_optical_interval> &intervals, double tolerance,
                        std::vector<dvs_event> &events, bool check_convergence = false) {
    size_t n = 0;
    int32_t accepted = 0;
    check(dvs_sensor_process_adaptive(sensor_.get(), intervals.data(), intervals.size(), tolerance,
                                      check_convergence ? 1 : 0, &accepted, &n));
    if (!accepted) {
      events.clear();
      return false;
    }
    read(n, events);
    return true;
  }
  int adaptive_cache_capacity() {
    int32_t k = 0;
    check(dvs_sensor_adaptive_capacity(sensor_.get(), &k));
    return k;
  }
  dvs_refinement_stats refinement_statistics() const {
    dvs_refinement_stats r{};
    check(dvs_sensor_refinement_stats(sensor_.get(), &r));
    return r;
  }
  dvs_receptor_probe last_convergence() const {
    dvs_receptor_probe r{};
    check(dvs_sensor_last_convergence(sensor_.get(), &r));
    return r;
  }
  void drain(std::vector<dvs_event> &events) {
    events.clear();
    std::vector<dvs_event> chunk(1 << 16);
    for (;;) {
      size_t got = 0;
      check(dvs_sensor_drain(sensor_.get(), chunk.data(), chunk.size(), &got));
      events.insert(events.end(), chunk.begin(), chunk.begin() + got);
      if (got < chunk.size()) break;
    }
  }
  dvs_sensor_stats stats() const {
    dvs_sensor_stats st{};
    check(dvs_sensor_stats_get(sensor_.get(), &st));
    return st;
  }
  std::size_t dropped_events() const { return stats().dropped; }
  std::size_t peak_queue() const { return stats().peak_queue; }
  dvs_sensor *get() const { return sensor_.get(); }

 private:
  friend class SensorBatch;
  void read(size_t n, std::vector<dvs_event> &events) {
    events.resize(n);
    size_t got = 0;
    if (n) check(dvs_sensor_read(sensor_.get(), events.data(), n, &got));
    events.resize(got);
  }
  struct Deleter {
    void operator()(dvs_sensor *s) const { dvs_sensor_destroy(s); }
  };
  std::shared_ptr<DeviceScene> scene_;
  std::unique_ptr<dvs_sensor, Deleter> sensor_;
};

class CamRayCaster {
 public:
  explicit CamRayCaster(std::shared_ptr<DeviceScene> scene) : scene_(std::move(scene)) {}
  void render_main(const dvs_optical_state &pose, std::vector<float> &light_frame, std::vector<float> &depth_map) {
    const size_t n = size_t(scene_->camera().width) * scene_->camera().height;
    light_frame.resize(n);
    depth_map.resize(n);
    check(dvs_cam_render(scene_->get(), &pose, light_frame.data(), depth_map.data()));
  }
  // Motion-blur exposure: all sub-exposure poses in one launch, accumulated
  // with the given weights in pose order (apps/main_cam_blur.cpp:64-77).
  void render_blur(const std::vector<dvs_optical_state> &poses, const std::vector<float> &weights,
                   std::vector<float> &image) {
    if (poses.size() != weights.size()) throw std::invalid_argument("one exposure weight per pose");
    image.resize(size_t(scene_->camera().width) * scene_->camera().height);
    check(dvs_cam_render_blur(scene_->get(), poses.data(), weights.data(), poses.size(), image.data()));
  }
  // The reference's call (src/cuda/cam_render.cu:16-28): camera_world is a
  // column-major 3x3 camera-to-world rotation, turned into a unit quaternion.
  void render_main(const dvs_float3 &origin, const float *camera_world, const dvs_float3 &light, float intensity,
                   std::vector<float> &light_frame, std::vector<float> &depth_map) {
    dvs_optical_state pose{};
    pose.position = origin;
    pose.light = light;
    pose.intensity = intensity;
    pose.rotation = quaternion_of(camera_world);
    render_main(pose, light_frame, depth_map);
  }

  // Unit quaternion (x, y, z, w) of a column-major rotation matrix
  // (Shepperd's method: branch on the largest of trace and diagonal).
  static dvs_float4 quaternion_of(const float *m) {
    auto R = [m](int r, int c) { return m[c * 3 + r]; };
    float q[4];  // x, y, z, w
    const float trace = R(0, 0) + R(1, 1) + R(2, 2);
    if (trace > 0) {
      float t = std::sqrt(trace + 1.0f);
      q[3] = 0.5f * t;
      t = 0.5f / t;
      q[0] = (R(2, 1) - R(1, 2)) * t;
      q[1] = (R(0, 2) - R(2, 0)) * t;
      q[2] = (R(1, 0) - R(0, 1)) * t;
    } else {
      int i = 0;
      if (R(1, 1) > R(0, 0)) i = 1;
      if (R(2, 2) > R(i, i)) i = 2;
      const int j = (i + 1) % 3, k = (j + 1) % 3;
      float t = std::sqrt(R(i, i) - R(j, j) - R(k, k) + 1.0f);
      q[i] = 0.5f * t;
      t = 0.5f / t;
      q[3] = (R(k, j) - R(j, k)) * t;
      q[j] = (R(j, i) + R(i, j)) * t;
      q[k] = (R(k, i) + R(i, k)) * t;
    }
    const float n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (n2 > 0) {
      const float n = std::sqrt(n2);
      for (float &v : q) v /= n;
    }
    dvs_float4 out{};
    out.x = q[0];
    out.y = q[1];
    out.z = q[2];
    out.w = q[3];
    return out;
  }

 private:
  std::shared_ptr<DeviceScene> scene_;
};

// Many DvsRayCasters over one scene geometry advanced together (dvs_batch_*):
// one persistent trace launch and one circuit launch per step, captured into a
// CUDA graph; each member's events are those it yields alone.  The members
// must outlive the batch.  No counterpart in the reference.
class SensorBatch {
 public:
  explicit SensorBatch(const std::vector<DvsRayCaster *> &members) : members_(members) {
    std::vector<dvs_sensor *> handles;
    for (DvsRayCaster *m : members) handles.push_back(m ? m->get() : nullptr);
    dvs_batch *b = nullptr;
    check(dvs_batch_create(handles.data(), handles.size(), &b));
    batch_.reset(b);
  }
  // intervals[m]: member m's next contiguous intervals (empty: it idles this
  // step); events[m] receives member m's ready events.
  void advance_many(const std::vector<std::vector<dvs_optical_interval>> &intervals,
                    std::vector<std::vector<dvs_event>> &events) {
    const size_t n = members_.size();
    if (intervals.size() != n) throw std::invalid_argument("one interval list per batch sensor");
    std::vector<const dvs_optical_interval *> ptr(n);
    std::vector<size_t> count(n), ready(n, 0);
    for (size_t m = 0; m < n; ++m) {
      ptr[m] = intervals[m].empty() ? nullptr : intervals[m].data();
      count[m] = intervals[m].size();
    }
    check(dvs_batch_process(batch_.get(), ptr.data(), count.data(), ready.data()));
    events.resize(n);
    for (size_t m = 0; m < n; ++m) {
      if (count[m]) members_[m]->read(ready[m], events[m]);
      else events[m].clear();
    }
  }
  dvs_batch_stats stats() const {
    dvs_batch_stats st{};
    check(dvs_batch_stats_get(batch_.get(), &st));
    return st;
  }

 private:
  struct Deleter {
    void operator()(dvs_batch *b) const { dvs_batch_destroy(b); }
  };
  std::vector<DvsRayCaster *> members_;
  std::unique_ptr<dvs_batch, Deleter> batch_;
};

}  // namespace dvs_gb300
