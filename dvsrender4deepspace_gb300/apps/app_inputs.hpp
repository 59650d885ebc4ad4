// Input loading shared by bin/dvs and bin/cam (apps/app_inputs.hpp of the
// reference): the scene bundle, the frame limit of the config, and the
// source_config.yaml / camera_used.yaml records in the output directory.
#pragma once
#include <algorithm>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

#include "app_cli.hpp"
#include "app_config.hpp"
#include "app_scene.hpp"

namespace dvs_app {

inline void load_app_inputs(const Options &opts, const Config &config, MeshBundle &mesh,
                            std::vector<FrameData> &frames) {
  std::string error;
  if (!opts.dem_path.empty() || !opts.traj_path.empty() || !opts.albedo_path.empty()) {
    if (opts.dem_path.empty() || opts.traj_path.empty())
      throw std::runtime_error("raster input requires both --dem and --traj");
    // DEM rasters are read through GDAL in the reference (src/tools/build_from_raster.cu)
    throw std::runtime_error("failed to load scene: raster (--dem) input needs GDAL, which this build does not "
                             "link; use a --scene_dir bundle (mesh_*.bin + frames.bin)");
  }
  if (!load_scene_bundle(opts.scene_dir, mesh, frames, &error)) throw std::runtime_error("failed to load scene: " + error);
  if (frames.empty()) throw std::runtime_error("empty trajectory");
  frames.resize(std::min(frames.size(), size_t(config.scene.frame_count)));
  std::filesystem::create_directories(opts.output_dir);
  const auto source = std::filesystem::absolute(opts.config_path);
  const auto destination = std::filesystem::absolute(std::filesystem::path(opts.output_dir) / "source_config.yaml");
  if (source.lexically_normal() != destination.lexically_normal())
    std::filesystem::copy_file(source, destination, std::filesystem::copy_options::overwrite_existing);
  std::ofstream out(std::filesystem::path(opts.output_dir) / "camera_used.yaml");
  if (!out) throw std::runtime_error("cannot write camera metadata");
  out << std::setprecision(9) << "source: " << source << "\nwidth: " << config.camera.width
      << "\nheight: " << config.camera.height << "\nfx: " << config.camera.fx << "\nfy: " << config.camera.fy
      << "\ncx: " << config.camera.cx << "\ncy: " << config.camera.cy
      << "\nsupersample_factor: " << config.scene.supersample_factor
      << "\npixel_centers: integer\nimage_axes: x_right_y_down\npose_axes: Blender_x_right_y_up_z_backward"
      << "\ndepth: mean_hit_ray_range_m; miss=-1"
      << "\ndistortion: not_implemented"
      << "\nphysics_calibration: generic_uncalibrated_optical_and_circuit_parameters\n";
}

}  // namespace dvs_app
