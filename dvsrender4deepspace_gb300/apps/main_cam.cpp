// bin/cam: drop-in for the reference's frame-camera app (apps/main_cam.cpp:22-114).
// Renders the trajectory at cam_fps and writes images/<t>.png (the 8-bit
// preview encoding) and depth/<t>.tif (float32 metres, -1 for misses),
// named by std::to_string of the frame time as the reference names them.
#include <cmath>
#include <filesystem>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "app_cli.hpp"
#include "app_config.hpp"
#include "app_inputs.hpp"
#include "app_trajectory.hpp"
#include "app_writers.hpp"
#include "dvs_gb300.hpp"

int main(int argc, char **argv) {
  try {
    if (argc <= 1) {
      dvs_app::Options::print_usage(argv[0]);
      return 1;
    }
    const dvs_app::Options opts(argc, argv);
    std::string error;
    dvs_app::Config config(opts.config_path, error);
    if (!error.empty()) throw std::runtime_error("failed to load config: " + error);
    dvs_app::MeshBundle mesh;
    std::vector<dvs_app::FrameData> frames;
    dvs_app::load_app_inputs(opts, config, mesh, frames);

    dvs_app::CameraTrajectory traj(frames, config.scene);
    auto scene = std::make_shared<dvs_gb300::DeviceScene>(mesh.vertices, mesh.normals, mesh.indices,
                                                          config.c_camera(), config.scene.supersample_factor,
                                                          config.c_hapke(), mesh.albedos.empty() ? nullptr : &mesh.albedos,
                                                          0, opts.bvh_flags());
    dvs_gb300::CamRayCaster raycaster(scene);
    const std::filesystem::path image_dir(opts.output_dir + "/images"), depth_dir(opts.output_dir + "/depth");
    std::filesystem::create_directories(image_dir);
    std::filesystem::create_directories(depth_dir);

    const size_t frame_count = std::min(frames.size(), size_t(config.scene.frame_count));
    if (frame_count == 0) throw std::runtime_error("no trajectory frames selected");
    const float end_time = float(dvs_app::frame_time(frames[frame_count - 1], config.scene.fps));
    const float start_time = float(dvs_app::frame_time(frames.front(), config.scene.fps));
    const size_t total_steps = size_t(std::ceil((double(end_time) - start_time) * config.scene.cam_fps));
    const float write_interval = 1.0f / config.scene.cam_fps;
    const int w = config.camera.width, h = config.camera.height;
    std::vector<float> light(size_t(w) * h), depth(size_t(w) * h);
    std::vector<uint8_t> bytes;
    size_t total_images = 0;
    for (size_t step = 0; step < total_steps; ++step) {
      const float current_time = start_time + step * write_interval;
      const dvs_app::TrajectoryState state = traj.evaluate(current_time);
      // column-major camera-to-world, as the reference passes Eigen's data()
      float world[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) world[c * 3 + r] = state.orientation(r, c);
      raycaster.render_main(dvs_float3{state.position.x, state.position.y, state.position.z}, world,
                            dvs_float3{state.light_direction.x, state.light_direction.y, state.light_direction.z},
                            state.light_intensity, light, depth);
      const std::string stem = std::to_string(current_time);
      dvs_app::render_float_to_png_bytes(light.data(), w, h, 0.0f, bytes);
      dvs_app::write_png_gray8((image_dir / (stem + ".png")).string(), bytes.data(), w, h);
      dvs_app::write_tiff_float32((depth_dir / (stem + ".tif")).string(), depth.data(), w, h);
      ++total_images;
    }
    std::cout << "Finished. Wrote " << total_images << " images to " << opts.output_dir << "\n";
    return 0;
  } catch (const std::exception &ex) {
    std::cerr << "Error: " << ex.what() << "\n";
    return 1;
  }
}
