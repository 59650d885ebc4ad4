// bin/cam_blur: drop-in for the reference's motion-blur camera
// (apps/main_cam_blur.cpp:20-91).  Each exposure of 1/cam_fps is cut into
// cells of blur_resolution seconds; the image is the duration-weighted sum of
// the cells' midpoint renders.  Here all cells of an exposure are traced in
// one multi-pose launch and summed on the device (dvs_cam_render_blur).
// Output: blur_images/<begin>.png (the 8-bit preview encoding).
#include <algorithm>
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
    const std::filesystem::path image_dir(opts.output_dir + "/blur_images");
    std::filesystem::create_directories(image_dir);

    const size_t frame_count = std::min(frames.size(), size_t(config.scene.frame_count));
    if (frame_count == 0) throw std::runtime_error("no trajectory frames selected");
    const float end_time = float(dvs_app::frame_time(frames[frame_count - 1], config.scene.fps));
    const float start_time = float(dvs_app::frame_time(frames.front(), config.scene.fps));
    const double interval = 1.0 / config.scene.cam_fps;
    const size_t exposures = size_t(std::ceil((double(end_time) - start_time) / interval));
    const int w = config.camera.width, h = config.camera.height;
    std::vector<float> image;
    std::vector<uint8_t> bytes;
    std::vector<dvs_optical_state> poses;
    std::vector<float> weights;
    size_t total_images = 0;
    for (size_t exposure = 0; exposure < exposures; ++exposure) {
      const double begin = start_time + exposure * interval;
      const double end = std::min(double(end_time), start_time + (exposure + 1) * interval);
      if (end <= begin) break;
      const size_t cells = size_t(std::ceil((end - begin) / config.scene.blur_resolution));
      poses.clear();
      weights.clear();
      for (size_t cell = 0; cell < cells; ++cell) {
        const double left = begin + cell * double(config.scene.blur_resolution);
        const double right = std::min(end, begin + (cell + 1) * double(config.scene.blur_resolution));
        const dvs_app::TrajectoryState state = traj.evaluate(float((left + right) * .5));
        float world[9];  // column-major, as the reference hands Eigen's data() to render_main
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) world[c * 3 + r] = state.orientation(r, c);
        dvs_optical_state pose{};
        pose.position = dvs_float3{state.position.x, state.position.y, state.position.z};
        pose.light = dvs_float3{state.light_direction.x, state.light_direction.y, state.light_direction.z};
        pose.intensity = state.light_intensity;
        pose.rotation = dvs_gb300::CamRayCaster::quaternion_of(world);
        poses.push_back(pose);
        weights.push_back(float((right - left) / (end - begin)));
      }
      raycaster.render_blur(poses, weights, image);
      dvs_app::render_float_to_png_bytes(image.data(), w, h, 0.0f, bytes);
      dvs_app::write_png_gray8((image_dir / (std::to_string(begin) + ".png")).string(), bytes.data(), w, h);
      ++total_images;
    }
    std::cout << "Finished. Wrote " << total_images << " images to " << opts.output_dir << "\n";
    return 0;
  } catch (const std::exception &ex) {
    std::cerr << "Error: " << ex.what() << "\n";
    return 1;
  }
}
