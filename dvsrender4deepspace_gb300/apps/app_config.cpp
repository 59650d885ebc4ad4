// Config loader of the drop-in apps: src/scene_types.cpp:9-345 semantics.
#include "app_config.hpp"

#include <cctype>
#include <charconv>
#include <cmath>
#include <fstream>
#include <limits>
#include <stdexcept>

namespace dvs_app {
namespace {

std::string strip(const std::string &s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  return s.substr(b, e - b);
}

// Cuts a trailing "# comment" that is not inside single or double quotes.
std::string cut_comment(const std::string &v) {
  char quote = 0;
  for (size_t i = 0; i < v.size(); ++i) {
    const char c = v[i];
    if (quote) {
      if (c == quote) quote = 0;
    } else if (c == '\'' || c == '"') {
      quote = c;
    } else if (c == '#') {
      return v.substr(0, i);
    }
  }
  return v;
}

template <typename T>
bool required(const std::unordered_map<std::string, std::string> &map, const char *section, const char *key, T &dst,
              std::string &err, bool (*convert)(const std::string &, T &)) {
  auto it = map.find(key);
  if (it == map.end()) {
    err = std::string("Missing key '") + key + "' in section '" + section + "'";
    return false;
  }
  if (!convert(it->second, dst)) {
    err = std::string("Invalid value for key '") + key + "' in section '" + section + "': '" + it->second + "'";
    return false;
  }
  return true;
}

}  // namespace

bool parse_yaml_to_map(const std::string &path, YamlMap &kv, std::string &err) {
  std::ifstream in(path);
  if (!in.is_open()) {
    err = "Cannot open file: " + path;
    return false;
  }
  std::string line, section;
  int number = 0;
  while (std::getline(in, line)) {
    ++number;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    size_t indent = 0;
    while (indent < line.size() && std::isspace(static_cast<unsigned char>(line[indent]))) ++indent;
    if (indent == line.size() || line[indent] == '#') continue;
    const size_t colon = line.find(':', indent);
    if (colon == std::string::npos) {
      err = "Line " + std::to_string(number) + ": missing colon";
      return false;
    }
    const std::string key = strip(line.substr(indent, colon - indent));
    if (key.empty()) {
      err = "Line " + std::to_string(number) + ": empty key";
      return false;
    }
    const std::string value = strip(cut_comment(colon + 1 < line.size() ? line.substr(colon + 1) : std::string()));
    if (indent == 0) {
      if (!value.empty()) {
        err = "Line " + std::to_string(number) + ": top-level key '" + key + "' has a value, expected a mapping";
        return false;
      }
      section = key;
      kv[section];
    } else {
      if (section.empty()) {
        err = "Line " + std::to_string(number) + ": key '" + key + "' without a parent section";
        return false;
      }
      kv[section][key] = value;
    }
  }
  return true;
}

bool safe_stoi(const std::string &s, int &out) {
  const char *b = s.data(), *e = s.data() + s.size();
  auto r = std::from_chars(b, e, out);
  return r.ec == std::errc{} && r.ptr == e;
}

bool safe_stof(const std::string &s, float &out) {
  const char *b = s.data(), *e = s.data() + s.size();
  auto r = std::from_chars(b, e, out);
  return r.ec == std::errc{} && r.ptr == e;
}

bool safe_stof_list(const std::string &s, std::vector<float> &out) {
  out.clear();
  if (s.size() < 2 || s.front() != '[' || s.back() != ']') return false;
  const std::string inner = s.substr(1, s.size() - 2);
  size_t pos = 0;
  while (true) {
    const size_t comma = inner.find(',', pos);
    const std::string item = strip(inner.substr(pos, comma == std::string::npos ? std::string::npos : comma - pos));
    float v;
    if (!safe_stof(item, v)) return false;
    out.push_back(v);
    if (comma == std::string::npos) break;
    pos = comma + 1;
  }
  return true;
}

Config::Config(const std::string &config_file, std::string &err) {
  YamlMap kv;
  if (!parse_yaml_to_map(config_file, kv, err)) return;
  for (const char *section : {"intrinsic", "physic", "scene"})
    if (kv.find(section) == kv.end()) {
      err = "Missing top-level section '" + std::string(section) + "'";
      return;
    }

  const auto &cam = kv["intrinsic"];
  if (!required(cam, "intrinsic", "width", camera.width, err, safe_stoi) ||
      !required(cam, "intrinsic", "height", camera.height, err, safe_stoi) ||
      !required(cam, "intrinsic", "fx", camera.fx, err, safe_stof) ||
      !required(cam, "intrinsic", "fy", camera.fy, err, safe_stof) ||
      !required(cam, "intrinsic", "cx", camera.cx, err, safe_stof) ||
      !required(cam, "intrinsic", "cy", camera.cy, err, safe_stof))
    return;

  const auto &ph = kv["physic"];
  if (!required(ph, "physic", "threshold_pos", physic.threshold_pos, err, safe_stof) ||
      !required(ph, "physic", "threshold_neg", physic.threshold_neg, err, safe_stof) ||
      !required(ph, "physic", "refractory_time", physic.refractory_time, err, safe_stof) ||
      !required(ph, "physic", "readout_latency", physic.readout_latency, err, safe_stof) ||
      !required(ph, "physic", "readout_bandwidth", physic.readout_bandwidth, err, safe_stof))
    return;
  // keys of the superseded phenomenological model are refused, not ignored
  for (const char *key : {"threshold_noise", "dark_current", "hpf_time_constant", "shot_intensity",
                          "photoreceptor_tau", "intensity_reference", "min_bandwidth_fraction", "leak_rate_hz",
                          "shot_noise_rate_hz", "shot_noise_bright_factor"})
    if (ph.count(key)) {
      err = std::string("removed physic key '") + key + "'; migrate to dimensioned parameters in docs/physical_sensor.md";
      return;
    }
  auto opt_f = [&](const char *key, float &v) {
    auto it = ph.find(key);
    if (it != ph.end() && !safe_stof(it->second, v))
      throw std::invalid_argument(std::string("invalid physic parameter: ") + key);
  };
  auto opt_i = [&](const char *key, int &v) {
    auto it = ph.find(key);
    if (it != ph.end() && !safe_stoi(it->second, v))
      throw std::invalid_argument(std::string("invalid physic parameter: ") + key);
  };
  PhysicConfig &p = physic;
  opt_f("threshold_std", p.threshold_std);
  opt_f("threshold_min", p.threshold_min);
  opt_f("wavelength_nm", p.wavelength_nm);
  opt_f("quantum_efficiency", p.quantum_efficiency);
  opt_f("pixel_pitch_um", p.pixel_pitch_um);
  opt_f("fill_factor", p.fill_factor);
  opt_f("f_number", p.f_number);
  opt_f("lens_transmission", p.lens_transmission);
  opt_f("radiance_scale", p.radiance_scale);
  opt_f("temperature_k", p.temperature_k);
  opt_f("subthreshold_kappa", p.subthreshold_kappa);
  opt_f("receptor_capacitance_f", p.receptor_capacitance_f);
  opt_f("reset_capacitance_f", p.reset_capacitance_f);
  opt_f("dark_current_a", p.dark_current_a);
  opt_f("reset_leakage_a", p.reset_leakage_a);
  opt_f("circuit_step", p.circuit_step);
  opt_i("photon_shot_noise", p.photon_shot_noise);
  opt_i("reset_thermal_noise", p.reset_thermal_noise);
  opt_i("random_seed", p.random_seed);
  opt_i("max_events_per_step", p.max_events_per_step);
  opt_i("readout_queue_capacity", p.readout_queue_capacity);
  for (float v : {p.threshold_pos, p.threshold_neg, p.threshold_std, p.threshold_min, p.refractory_time,
                  p.readout_bandwidth, p.readout_latency, p.wavelength_nm, p.quantum_efficiency, p.pixel_pitch_um,
                  p.fill_factor, p.f_number, p.lens_transmission, p.radiance_scale, p.temperature_k,
                  p.subthreshold_kappa, p.receptor_capacitance_f, p.reset_capacitance_f, p.dark_current_a,
                  p.reset_leakage_a, p.circuit_step})
    if (!std::isfinite(v) || v < 0) {
      err = "physic values must be finite and nonnegative";
      return;
    }
  if (p.threshold_pos <= 0 || p.threshold_neg <= 0 || p.threshold_min <= 0 || p.wavelength_nm <= 0 ||
      p.pixel_pitch_um <= 0 || p.f_number <= 0 || p.temperature_k <= 0 || p.subthreshold_kappa <= 0 ||
      p.subthreshold_kappa > 1 || p.receptor_capacitance_f <= 0 || p.reset_capacitance_f <= 0 ||
      p.circuit_step <= 0 || p.quantum_efficiency > 1 || p.fill_factor > 1 || p.lens_transmission > 1 ||
      p.photon_shot_noise < 0 || p.photon_shot_noise > 1 || p.reset_thermal_noise < 0 ||
      p.reset_thermal_noise > 1 || p.random_seed < 0 || p.max_events_per_step < 1 || p.max_events_per_step > 64 ||
      p.readout_queue_capacity < 1) {
    err = "invalid optical/circuit model parameter range";
    return;
  }

  const auto &sc = kv["scene"];
  if (!required(sc, "scene", "frame_count", scene.frame_count, err, safe_stoi) ||
      !required(sc, "scene", "fps", scene.fps, err, safe_stof) ||
      !required(sc, "scene", "imu_fps", scene.imu_fps, err, safe_stof) ||
      !required(sc, "scene", "cam_fps", scene.cam_fps, err, safe_stof) ||
      !required(sc, "scene", "time_resolution", scene.time_resolution, err, safe_stof) ||
      !required(sc, "scene", "supersample_factor", scene.supersample_factor, err, safe_stoi) ||
      !required(sc, "scene", "blur_resolution", scene.blur_resolution, err, safe_stof))
    return;
  scene.translation = {0, 0, 0};
  scene.rotation = {0, 0, 0};
  for (auto kvp : {std::make_pair("translation", &scene.translation), std::make_pair("rotation", &scene.rotation)}) {
    auto it = sc.find(kvp.first);
    if (it != sc.end() && (!safe_stof_list(it->second, *kvp.second) || kvp.second->size() != 3)) {
      err = std::string("scene.") + kvp.first + " must have three numbers";
      return;
    }
    for (float v : *kvp.second)
      if (!std::isfinite(v)) {
        err = "nonfinite extrinsics";
        return;
      }
  }
  for (float v : {camera.fx, camera.fy, camera.cx, camera.cy, scene.fps, scene.time_resolution, scene.cam_fps,
                  scene.imu_fps, scene.blur_resolution})
    if (!std::isfinite(v)) {
      err = "nonfinite camera or scene parameter";
      return;
    }
  if (camera.width <= 0 || camera.height <= 0 || camera.width > 32767 || camera.height > 32767 || camera.fx <= 0 ||
      camera.fy <= 0 || scene.frame_count < 2 || scene.fps <= 0 || scene.time_resolution <= 0 ||
      scene.cam_fps <= 0 || scene.imu_fps <= 0 || scene.blur_resolution <= 0 || scene.supersample_factor < 1) {
    err = "invalid scene or camera range";
    return;
  }
  const double samples =
      double(camera.width) * camera.height * scene.supersample_factor * scene.supersample_factor;
  if (samples > std::numeric_limits<int>::max()) {
    err = "too many aperture samples";
    return;
  }

  const auto &hp = kv["hapke"];
  if (!required(hp, "hapke", "b", hapke.b, err, safe_stof) || !required(hp, "hapke", "c", hapke.c, err, safe_stof) ||
      !required(hp, "hapke", "hS", hapke.hS, err, safe_stof) ||
      !required(hp, "hapke", "hC", hapke.hC, err, safe_stof) ||
      !required(hp, "hapke", "thetap", hapke.thetap, err, safe_stof) ||
      !required(hp, "hapke", "w", hapke.w, err, safe_stof) ||
      !required(hp, "hapke", "B_S0", hapke.B_S0, err, safe_stof) ||
      !required(hp, "hapke", "B_C0", hapke.B_C0, err, safe_stof) ||
      !required(hp, "hapke", "phi", hapke.phi, err, safe_stof))
    return;
  const HapkeConfig &h = hapke;
  for (float v : {h.b, h.c, h.hS, h.hC, h.thetap, h.w, h.B_S0, h.B_C0, h.phi})
    if (!std::isfinite(v)) {
      err = "nonfinite Hapke parameter";
      return;
    }
  const float half_pi = 3.14159265358979323846f / 2;
  if (h.b < 0 || h.b >= 1 || h.c < -1 || h.c > 1 || h.hS < 0 || h.hC < 0 || h.thetap < 0 || h.thetap >= half_pi ||
      h.w < 0 || h.w > 1 || h.B_S0 < 0 || h.B_C0 < 0 || h.phi < 0 ||
      1.209f * std::pow(h.phi, 2.0f / 3.0f) >= 1) {
    err = "invalid Hapke parameter range";
    return;
  }
}

dvs_camera Config::c_camera() const {
  return dvs_camera{camera.width, camera.height, camera.fx, camera.fy, camera.cx, camera.cy};
}

dvs_physic Config::c_physic() const {
  const PhysicConfig &p = physic;
  dvs_physic o{};
  o.threshold_pos = p.threshold_pos;
  o.threshold_neg = p.threshold_neg;
  o.refractory_time = p.refractory_time;
  o.readout_bandwidth = p.readout_bandwidth;
  o.readout_latency = p.readout_latency;
  o.threshold_std = p.threshold_std;
  o.threshold_min = p.threshold_min;
  o.wavelength_nm = p.wavelength_nm;
  o.quantum_efficiency = p.quantum_efficiency;
  o.pixel_pitch_um = p.pixel_pitch_um;
  o.fill_factor = p.fill_factor;
  o.f_number = p.f_number;
  o.lens_transmission = p.lens_transmission;
  o.radiance_scale = p.radiance_scale;
  o.temperature_k = p.temperature_k;
  o.subthreshold_kappa = p.subthreshold_kappa;
  o.receptor_capacitance_f = p.receptor_capacitance_f;
  o.reset_capacitance_f = p.reset_capacitance_f;
  o.dark_current_a = p.dark_current_a;
  o.reset_leakage_a = p.reset_leakage_a;
  o.circuit_step = p.circuit_step;
  o.photon_shot_noise = p.photon_shot_noise;
  o.reset_thermal_noise = p.reset_thermal_noise;
  o.random_seed = p.random_seed;
  o.max_events_per_step = p.max_events_per_step;
  o.readout_queue_capacity = p.readout_queue_capacity;
  return o;
}

dvs_hapke Config::c_hapke() const {
  return dvs_hapke{hapke.b, hapke.c, hapke.hS, hapke.hC, hapke.thetap, hapke.w, hapke.B_S0, hapke.B_C0, hapke.phi};
}

}  // namespace dvs_app
