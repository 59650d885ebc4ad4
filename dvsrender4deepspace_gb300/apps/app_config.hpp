// YAML configuration of the drop-in apps (src/scene_types.cpp:9-345,
// include/dvs/scene_types.hpp:61-111): the intrinsic / physic / scene / hapke
// blocks, the same required and optional keys, defaults, range checks and
// error texts, so a reference config file loads unchanged.
#pragma once
#include <string>
#include <unordered_map>
#include <vector>

#include "dvs_gb300.h"

namespace dvs_app {

struct CameraConfig {
  int width = 0, height = 0;
  float fx = 0, fy = 0, cx = 0, cy = 0;
};

// Defaults of include/dvs/scene_types.hpp:61-77.
struct PhysicConfig {
  float threshold_pos = .3f, threshold_neg = .3f, refractory_time = .0002f;
  float readout_bandwidth = 5e6f, readout_latency = 0;
  float threshold_std = 0.03f, threshold_min = 0.01f;
  float wavelength_nm = 550, quantum_efficiency = .3f, pixel_pitch_um = 15;
  float fill_factor = .2f, f_number = 2, lens_transmission = .8f;
  float radiance_scale = .001f;
  float temperature_k = 300, subthreshold_kappa = .8f;
  float receptor_capacitance_f = 1e-15f;
  float reset_capacitance_f = 20e-15f, dark_current_a = 1e-18f;
  float reset_leakage_a = 0, circuit_step = 1e-6f;
  int photon_shot_noise = 1, reset_thermal_noise = 0;
  int random_seed = 114514, max_events_per_step = 16;
  int readout_queue_capacity = 1000000;
};

struct SceneConfig {
  int frame_count = 0;
  float fps = 0, imu_fps = 0, cam_fps = 0;
  float time_resolution = 0, blur_resolution = 0;
  int supersample_factor = 0;
  std::vector<float> translation, rotation;
};

// Defaults of include/dvs/scene_types.hpp:88-98.
struct HapkeConfig {
  float b = 0.24f, c = 0.305f, hS = 0.08f, hC = 1.0f;
  float thetap = 26.0f * 3.14159265358979323846f / 180.0f;
  float w = 0.324f, B_S0 = 2.42f, B_C0 = 0.0f, phi = 0.3f;
};

class Config {
 public:
  CameraConfig camera;
  PhysicConfig physic;
  SceneConfig scene;
  HapkeConfig hapke;

  // On failure err holds the reference's message and the fields are partial.
  Config(const std::string &config_file, std::string &err);

  dvs_camera c_camera() const;
  dvs_physic c_physic() const;
  dvs_hapke c_hapke() const;
};

using YamlMap = std::unordered_map<std::string, std::unordered_map<std::string, std::string>>;
// Two-level "section: / key: value" YAML subset (scene_types.cpp:9-125).
bool parse_yaml_to_map(const std::string &path, YamlMap &kv, std::string &err);
bool safe_stoi(const std::string &s, int &out);
bool safe_stof(const std::string &s, float &out);
bool safe_stof_list(const std::string &s, std::vector<float> &out);

}  // namespace dvs_app
