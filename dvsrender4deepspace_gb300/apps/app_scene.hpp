// Scene bundle and trajectory-frame loaders of the drop-in apps
// (src/scene_data.cpp:93-282): mesh_vertices.bin / mesh_normals.bin /
// mesh_indices.bin (N x 3 float32, float32, uint32) and frames.bin (24
// float32 per frame: seconds, camera origin, row-major 4x4 camera-to-world,
// light direction, light intensity), or a text trajectory of
// "frame x y z qx qy qz qw lx ly lz intensity" lines.
#pragma once
#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include "app_math.hpp"

namespace dvs_app {

struct FrameData {
  int frame_index = 0;
  double timestamp_seconds = std::numeric_limits<double>::quiet_NaN();
  V3 camera_origin;
  M3 camera_world;
  V3 light_dir;
  float light_intensity = 0.0f;
};

// Binary frames store seconds; text trajectories store frame indices
// (include/dvs/scene_types.hpp:52-55).
inline double frame_time(const FrameData &f, double fps) {
  return std::isnan(f.timestamp_seconds) ? f.frame_index / fps : f.timestamp_seconds;
}

struct MeshBundle {
  std::vector<float> vertices, normals;  // n_vertices x 3
  std::vector<uint32_t> indices;         // n_triangles x 3
  std::vector<float> albedos;            // empty, or n_vertices
};

bool load_mesh_data(const std::string &dir, MeshBundle &out, std::string *err);
bool load_frames_from_binary(const std::string &dir, std::vector<FrameData> &out, std::string *err);
bool load_frames_from_text(const std::string &path, std::vector<FrameData> &out, std::string *err);
// Directory bundle: mesh + frames.bin (src/scene_data.cpp:195-236).
bool load_scene_bundle(const std::string &dir, MeshBundle &mesh, std::vector<FrameData> &frames, std::string *err);

}  // namespace dvs_app
