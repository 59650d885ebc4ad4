// C-ABI of the apps' host inputs (config, frames.bin, trajectory), compiled
// into libdvs_gb300.so so that any host (the Python package, a maintainer's
// own driver) evaluates exactly the trajectory bin/dvs and bin/cam use.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <new>
#include <string>
#include <vector>

#include "app_config.hpp"
#include "app_scene.hpp"
#include "app_trajectory.hpp"
#include "dvs_gb300.h"

int dvsgb_set_error(int code, const char *message);  // csrc/capi.cu

struct dvs_trajectory {
  dvs_app::CameraTrajectory traj;
};

namespace {

dvs_app::SceneConfig to_scene(const dvs_scene_config &c) {
  dvs_app::SceneConfig s;
  s.frame_count = c.frame_count;
  s.fps = c.fps;
  s.imu_fps = c.imu_fps;
  s.cam_fps = c.cam_fps;
  s.time_resolution = c.time_resolution;
  s.blur_resolution = c.blur_resolution;
  s.supersample_factor = c.supersample_factor;
  s.translation.assign(c.translation, c.translation + 3);
  s.rotation.assign(c.rotation, c.rotation + 3);
  return s;
}

dvs_app::FrameData to_frame(const dvs_frame &f) {
  dvs_app::FrameData o;
  o.frame_index = f.frame_index;
  o.timestamp_seconds = f.timestamp_seconds;
  o.camera_origin = dvs_app::V3(f.camera_origin[0], f.camera_origin[1], f.camera_origin[2]);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o.camera_world.m[r][c] = f.camera_world[3 * r + c];
  o.light_dir = dvs_app::V3(f.light_dir[0], f.light_dir[1], f.light_dir[2]);
  o.light_intensity = f.light_intensity;
  return o;
}

}  // namespace

extern "C" {

int dvs_config_load(const char *path, dvs_camera *camera, dvs_physic *physic, dvs_hapke *hapke,
                    dvs_scene_config *scene) {
  if (!path) return dvsgb_set_error(DVS_ERR_INVALID, "null config path");
  try {
    std::string err;
    dvs_app::Config config(path, err);
    if (!err.empty()) return dvsgb_set_error(DVS_ERR_INVALID, err.c_str());
    if (camera) *camera = config.c_camera();
    if (physic) *physic = config.c_physic();
    if (hapke) *hapke = config.c_hapke();
    if (scene) {
      dvs_scene_config s{};
      s.frame_count = config.scene.frame_count;
      s.fps = config.scene.fps;
      s.imu_fps = config.scene.imu_fps;
      s.cam_fps = config.scene.cam_fps;
      s.time_resolution = config.scene.time_resolution;
      s.blur_resolution = config.scene.blur_resolution;
      s.supersample_factor = config.scene.supersample_factor;
      for (int i = 0; i < 3; ++i) {
        s.translation[i] = config.scene.translation[size_t(i)];
        s.rotation[i] = config.scene.rotation[size_t(i)];
      }
      *scene = s;
    }
    return DVS_OK;
  } catch (const std::exception &e) {
    return dvsgb_set_error(DVS_ERR_INVALID, e.what());
  }
}

int dvs_frames_load(const char *bundle_dir, dvs_frame *frames, size_t capacity, size_t *n_frames) {
  if (!bundle_dir || !n_frames) return dvsgb_set_error(DVS_ERR_INVALID, "null argument");
  std::vector<dvs_app::FrameData> in;
  std::string err;
  if (!dvs_app::load_frames_from_binary(bundle_dir, in, &err)) return dvsgb_set_error(DVS_ERR_INVALID, err.c_str());
  *n_frames = in.size();
  if (!frames) return DVS_OK;
  const size_t n = std::min(capacity, in.size());
  for (size_t i = 0; i < n; ++i) {
    dvs_frame f{};
    f.frame_index = in[i].frame_index;
    f.timestamp_seconds = in[i].timestamp_seconds;
    for (int d = 0; d < 3; ++d) {
      f.camera_origin[d] = in[i].camera_origin[d];
      f.light_dir[d] = in[i].light_dir[d];
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) f.camera_world[3 * r + c] = in[i].camera_world.m[r][c];
    f.light_intensity = in[i].light_intensity;
    frames[i] = f;
  }
  if (capacity < in.size()) return dvsgb_set_error(DVS_ERR_OUTPUT_SMALL, "frame buffer smaller than frames.bin");
  return DVS_OK;
}

int dvs_trajectory_create(const dvs_frame *frames, size_t n_frames, const dvs_scene_config *scene,
                          dvs_trajectory **out) {
  if (!out) return dvsgb_set_error(DVS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!scene || (!frames && n_frames)) return dvsgb_set_error(DVS_ERR_INVALID, "null argument");
  try {
    std::vector<dvs_app::FrameData> in(n_frames);
    for (size_t i = 0; i < n_frames; ++i) in[i] = to_frame(frames[i]);
    *out = new dvs_trajectory{dvs_app::CameraTrajectory(in, to_scene(*scene))};
    return DVS_OK;
  } catch (const std::exception &e) {
    return dvsgb_set_error(DVS_ERR_INVALID, e.what());
  }
}

int dvs_trajectory_destroy(dvs_trajectory *t) {
  delete t;
  return DVS_OK;
}

int dvs_trajectory_range(const dvs_trajectory *t, float *start_time, float *end_time) {
  if (!t) return dvsgb_set_error(DVS_ERR_INVALID, "null trajectory");
  if (start_time) *start_time = t->traj.start_time();
  if (end_time) *end_time = t->traj.end_time();
  return DVS_OK;
}

int dvs_trajectory_evaluate(const dvs_trajectory *t, float time, dvs_optical_state *state, float *orientation9) {
  if (!t || !state) return dvsgb_set_error(DVS_ERR_INVALID, "null argument");
  const dvs_app::TrajectoryState s = t->traj.evaluate(time);
  *state = dvs_app::to_optical_state(s);
  if (orientation9)
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) orientation9[3 * r + c] = s.orientation(r, c);
  return DVS_OK;
}

}  // extern "C"
