// Scene bundle loaders: src/scene_data.cpp:30-282 semantics and messages.
#include "app_scene.hpp"

#include <cctype>
#include <cmath>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>

namespace dvs_app {
namespace {

template <typename T>
bool read_raw(const std::filesystem::path &path, const char *kind, std::vector<T> *out, std::string *err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    if (err) *err = "failed to open " + path.string();
    return false;
  }
  in.seekg(0, std::ios::end);
  const std::streamoff size = in.tellg();
  in.seekg(0, std::ios::beg);
  if (size < 0 || size % std::streamoff(sizeof(T)) != 0) {
    if (err) *err = std::string("invalid ") + kind + " binary size for " + path.string();
    return false;
  }
  out->resize(size_t(size / std::streamoff(sizeof(T))));
  in.read(reinterpret_cast<char *>(out->data()), size);
  if (!in) {
    if (err) *err = "failed to read " + path.string();
    return false;
  }
  return true;
}

std::string trim(const std::string &s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  return s.substr(b, e - b);
}

}  // namespace

bool load_mesh_data(const std::string &dir_s, MeshBundle &out, std::string *err) {
  const std::filesystem::path dir(dir_s);
  if (!read_raw(dir / "mesh_vertices.bin", "f32", &out.vertices, err) ||
      !read_raw(dir / "mesh_normals.bin", "f32", &out.normals, err) ||
      !read_raw(dir / "mesh_indices.bin", "u32", &out.indices, err))
    return false;
  if (out.vertices.size() % 3 || out.normals.size() % 3 || out.indices.size() % 3) {
    if (err) *err = "mesh binaries must be Nx3";
    return false;
  }
  if (out.vertices.empty() || out.indices.empty() || out.vertices.size() != out.normals.size()) {
    if (err) *err = "mesh requires nonempty vertices/triangles and matching normals";
    return false;
  }
  const size_t nv = out.vertices.size() / 3;
  for (uint32_t i : out.indices)
    if (i >= nv) {
      if (err) *err = "mesh index outside vertex array";
      return false;
    }
  for (float v : out.vertices)
    if (!std::isfinite(v)) {
      if (err) *err = "nonfinite mesh vertex";
      return false;
    }
  for (float v : out.normals)
    if (!std::isfinite(v)) {
      if (err) *err = "nonfinite mesh normal";
      return false;
    }
  return true;
}

bool load_frames_from_binary(const std::string &dir, std::vector<FrameData> &out, std::string *err) {
  constexpr size_t kStride = 24;
  std::vector<float> raw;
  if (!read_raw(std::filesystem::path(dir) / "frames.bin", "f32", &raw, err)) return false;
  if (raw.size() % kStride) {
    if (err) *err = "frames.bin has invalid stride";
    return false;
  }
  out.resize(raw.size() / kStride);
  for (size_t i = 0; i < out.size(); ++i) {
    const float *r = raw.data() + i * kStride;
    FrameData f;
    f.timestamp_seconds = r[0];
    f.camera_origin = V3(r[1], r[2], r[3]);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) f.camera_world.m[a][b] = r[4 + 4 * a + b];  // top-left of a row-major 4x4
    f.light_dir = V3(r[20], r[21], r[22]);
    f.light_intensity = r[23];
    out[i] = f;
  }
  return true;
}

bool load_frames_from_text(const std::string &path, std::vector<FrameData> &out, std::string *err) {
  if (!std::filesystem::exists(path)) {
    if (err) *err = "file does not exist: " + path;
    return false;
  }
  std::ifstream in(path);
  if (!in) {
    if (err) *err = "failed to open " + path;
    return false;
  }
  std::string line;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.empty()) continue;
    std::istringstream ss(line);
    FrameData f;
    float qx, qy, qz, qw;
    if (!(ss >> f.frame_index >> f.camera_origin.x >> f.camera_origin.y >> f.camera_origin.z >> qx >> qy >> qz >> qw >>
          f.light_dir.x >> f.light_dir.y >> f.light_dir.z >> f.light_intensity)) {
      if (err) *err = "failed to parse camera orientation in line: " + line;
      return false;
    }
    f.camera_world = qmatrix(Quat(qw, qx, qy, qz));
    out.push_back(f);
  }
  return true;
}

bool load_scene_bundle(const std::string &dir, MeshBundle &mesh, std::vector<FrameData> &frames, std::string *err) {
  if (!load_mesh_data(dir, mesh, err)) return false;
  std::cout << "Loaded mesh with " << mesh.vertices.size() / 3 << " vertices, " << mesh.normals.size() / 3
            << " normals, and " << mesh.indices.size() / 3 << " triangles" << std::endl;
  if (!load_frames_from_binary(dir, frames, err)) return false;
  if (frames.empty()) {
    if (err) *err = "frames.bin is empty";
    return false;
  }
  return true;
}

}  // namespace dvs_app
