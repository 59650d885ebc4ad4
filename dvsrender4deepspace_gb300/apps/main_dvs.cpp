// bin/dvs: drop-in for the reference's event app (apps/main_dvs.cpp:37-171).
// Same command line, config, inputs, horizon batching, adaptive-solver
// selection and retry, write cadence, outputs (events.bin or events.h5,
// sensor_config.yaml, sensor_model.txt) and messages; the scene, sensor and
// readout run on the GB300 path through the dvs_gb300 C-ABI.
#include <algorithm>
#include <cmath>
#include <filesystem>
#include <fstream>
#include <iomanip>
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

namespace {

constexpr double kDefaultOpticalLogTolerance = 1e-2;        // include/dvs/optical_sampler.hpp:6
constexpr double kOpticalVoltageThresholdFraction = 1e-3;   // include/dvs/optical_sampler.hpp:7

std::unique_ptr<dvs_app::EventStreamWriter> make_event_writer(const dvs_app::Options &opts) {
  if (opts.event_format == "hdf5")
    return std::make_unique<dvs_app::Hdf5EventStreamWriter>(opts.output_dir + "/events.h5");
  if (opts.event_format == "bin")
    return std::make_unique<dvs_app::BinaryEventStreamWriter>(opts.output_dir + "/events.bin");
  throw std::runtime_error("unsupported event format: " + opts.event_format);
}

}  // namespace

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

    // physical effects are on, as in the reference's default build
    bool adaptive = opts.event_solver == "adaptive-optics" ||
                    (opts.event_solver == "auto" && opts.event_format == "hdf5" && config.physic.refractory_time > 0);
    if (adaptive && opts.event_format != "hdf5")
      throw std::runtime_error(
          "adaptive optics exports HDF5 x/y/t/p; per-event auxiliary binary depth requires --solver native");
    if (adaptive && opts.circuit == "fp32-philox")
      throw std::runtime_error("the adaptive solver keeps the XORWOW noise stream: use --circuit fp32 or --solver native");
    dvs_app::MeshBundle mesh;
    std::vector<dvs_app::FrameData> frames;
    dvs_app::load_app_inputs(opts, config, mesh, frames);

    dvs_app::CameraTrajectory traj(frames, config.scene);
    auto scene = std::make_shared<dvs_gb300::DeviceScene>(mesh.vertices, mesh.normals, mesh.indices,
                                                          config.c_camera(), config.scene.supersample_factor,
                                                          config.c_hapke(), mesh.albedos.empty() ? nullptr : &mesh.albedos,
                                                          0, opts.bvh_flags());
    dvs_sensor_options options;
    dvs_sensor_options_default(&options);
    options.circuit_precision = opts.circuit_precision();
    dvs_gb300::DvsRayCaster raycaster(scene, config.c_physic(), &options);
    std::filesystem::create_directories(opts.output_dir);
    std::unique_ptr<dvs_app::EventStreamWriter> events_out = make_event_writer(opts);

    const size_t frame_count = std::min(frames.size(), size_t(config.scene.frame_count));
    if (frame_count == 0) throw std::runtime_error("no trajectory frames selected");
    const float end_time = float(dvs_app::frame_time(frames[frame_count - 1], config.scene.fps));
    const float start_time = float(dvs_app::frame_time(frames.front(), config.scene.fps));
    const size_t total_steps = size_t(std::ceil((double(end_time) - double(start_time)) /
                                                double(config.scene.time_resolution)));

    std::vector<dvs_event> events, events_buffer;
    double next_write_time = start_time;
    const float write_interval = 1.0f / config.scene.imu_fps;

    dvs_app::TrajectoryState previous_state = traj.evaluate(start_time);
    raycaster.initialize(dvs_app::to_optical_state(previous_state), start_time);
    std::cout << "Initialized continuous photocurrent/circuit state from scene rays.\n";
    double previous_time = start_time;
    // horizons per launch: 200 adaptive / 64 native, bounded by the pixel
    // event capacity over the refractory time (apps/main_dvs.cpp:94-98)
    unsigned batch = adaptive ? 200 : 64;
    if (config.physic.refractory_time <= 0) {
      batch = 1;
    } else {
      const double cap = std::max(1.0, (config.physic.max_events_per_step - 2) * double(config.physic.refractory_time) /
                                           config.scene.time_resolution);
      batch = std::max(1U, std::min(batch, unsigned(cap)));
    }
    double next_check = start_time;
    size_t step = 0;
    std::vector<dvs_optical_interval> intervals;
    intervals.reserve(batch);
    while (step < total_steps) {
      const size_t first_step = step;
      const double first_time = previous_time;
      const dvs_app::TrajectoryState first_state = previous_state;
      intervals.clear();
      for (unsigned j = 0; j < batch && step < total_steps; ++j) {
        const double time = std::min(double(end_time), double(start_time) + double(++step) *
                                                                                double(config.scene.time_resolution));
        if (time <= previous_time) break;
        const dvs_app::TrajectoryState current = traj.evaluate(float(time));
        intervals.push_back(dvs_optical_interval{dvs_app::to_optical_state(previous_state),
                                                 dvs_app::to_optical_state(current), previous_time, time});
        previous_state = current;
        previous_time = time;
      }
      if (intervals.empty()) break;
      if (adaptive) {
        const bool check = first_time >= next_check;
        if (!raycaster.advance_adaptive(intervals, kDefaultOpticalLogTolerance, events, check)) {
          if (batch > 1) {  // rejected window: retry it in halves
            batch = std::max(1U, batch / 2);
            step = first_step;
            previous_time = first_time;
            previous_state = first_state;
            continue;
          }
          raycaster.advance_many(intervals, events);
        }
        if (check) next_check = previous_time + .25;
      } else {
        raycaster.advance_many(intervals, events);
      }
      events_buffer.insert(events_buffer.end(), events.begin(), events.end());
      events.clear();
      if (previous_time >= next_write_time) {
        next_write_time = previous_time + write_interval;
        events_out->append(std::move(events_buffer));
        events_buffer.clear();
      }
    }
    if (!events_buffer.empty()) {
      events_out->append(std::move(events_buffer));
      events_buffer.clear();
    }
    // finish the last interval and flush the transport backlog
    raycaster.drain(events);
    const double output_end =
        events.empty() ? double(end_time) : std::max(double(end_time), double(events.back().timestamp));
    events_out->append(std::move(events));
    events_out->close(output_end);
    {
      std::ifstream source_config(opts.config_path);
      std::ofstream copied_config(opts.output_dir + "/sensor_config.yaml");
      copied_config << source_config.rdbuf();
    }
    std::ofstream meta(opts.output_dir + "/sensor_model.txt");
    meta << std::setprecision(12) << "model=ray_photocurrent_circuit_v2\n"
         << "timestamp="
         << (opts.event_format == "hdf5" ? "int64_microseconds_transport_completion"
                                         : "float32_seconds_transport_completion")
         << "\n"
         << "config=" << opts.config_path << "\n"
         << "random_seed=" << config.physic.random_seed << "\n"
         << "dropped_readout_events=" << raycaster.dropped_events() << "\n"
         << "peak_readout_queue=" << raycaster.peak_queue() << "\n"
         << "physical_effects=on\n"
         << "photoreceptor=nonlinear_current_balance\n"
         << "optical_sampling="
         << (adaptive ? "adaptive_direct_ray_nodes_with_native_cell_fallback" : "midpoint_rays_within_circuit_cells")
         << "\n"
         << "optical_log_tolerance=" << (adaptive ? kDefaultOpticalLogTolerance : 0) << "\n"
         << "leaf_voltage_error_threshold_fraction=" << (adaptive ? kOpticalVoltageThresholdFraction : 0) << "\n"
         << "optical_cache_capacity=" << (adaptive ? raycaster.adaptive_cache_capacity() : 0) << "\n"
         << "camera_width=" << config.camera.width << "\ncamera_height=" << config.camera.height << "\n"
         << "fx=" << config.camera.fx << "\nfy=" << config.camera.fy << "\ncx=" << config.camera.cx
         << "\ncy=" << config.camera.cy << "\n"
         << "spatial_grid=" << config.scene.supersample_factor << "\n"
         << "distortion=ideal_pinhole_not_hardware_calibration\n"
         << "physics_calibration=generic_uncalibrated\n"
         << "photon_noise=charge_count_tau_leap\n"
         << "circuit_step_seconds=" << config.physic.circuit_step << "\n"
         << "radiance_scale=" << config.physic.radiance_scale << "\n"
         << "readout_queue=on\n";
    std::cout << "Readout dropped " << raycaster.dropped_events() << " events; peak queue " << raycaster.peak_queue()
              << "\n";
    std::cout << "Finished. Wrote " << events_out->event_count() << " events to " << events_out->path() << "\n";
    return 0;
  } catch (const std::exception &ex) {
    std::cerr << "Error: " << ex.what() << "\n";
    return 1;
  }
}
