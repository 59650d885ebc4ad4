// Command line of bin/dvs and bin/cam (include/tools/cli.hpp:9-101): the same
// flags, aliases, defaults, usage text and errors.
#pragma once
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>

namespace dvs_app {

class Options {
 public:
  std::string scene_dir, dem_path, albedo_path, traj_path;
  std::string output_dir = "./output";
  std::string config_path = "./config/davis346.yaml";
  std::string event_format = "bin";
  std::string event_solver = "auto";
  // GB300 additions (no reference counterpart): BVH format and pixel-circuit arithmetic
  std::string bvh = "fp32";        // fp32 | half | watertight | half+watertight
  std::string circuit = "fp64";    // fp64 | fp32 | fp32-philox

  int bvh_flags() const {  // dvs_bvh_params.precision
    return (bvh == "half" || bvh == "half+watertight" ? 1 : 0) |
           (bvh == "watertight" || bvh == "half+watertight" ? 2 : 0);
  }
  int circuit_precision() const { return circuit == "fp32" ? 1 : circuit == "fp32-philox" ? 2 : 0; }

  static void print_usage(const char *prog) {
    std::cout << "Usage: " << prog << "[options]\n"
              << "Options:\n"
              << "  --scene_dir <path>         path to scene bundle directory\n"
              << "  --dem <path>               path to DEM file (optional)\n"
              << "  --albedo <path>            path to albedo file (optional)\n"
              << "  --traj <path>              path to camera trajectory file (optional)\n"
              << "  --output <path>            output images file (default: ./)\n"
              << "  --config <path>            path to YAML config file (default: ./config/davis346.yaml)\n"
              << "  --event_format <bin|hdf5>  event stream output format (default: bin)\n"
              << "  --solver <auto|native|adaptive-optics>  auto selects adaptive optics for physical HDF5 output\n"
              << "  --bvh <fp32|half|watertight|half+watertight>  BVH child bounds and triangle test (default: fp32)\n"
              << "  --circuit <fp64|fp32|fp32-philox>  pixel-circuit arithmetic and noise stream (default: fp64)"
              << std::endl;
  }

  Options(int argc, char **argv) {
    for (int i = 1; i < argc; ++i) {
      const std::string arg = argv[i];
      auto value = [&](const char *key) -> std::string {
        if (i + 1 >= argc) throw std::runtime_error(std::string("missing value for ") + key);
        return std::string(argv[++i]);
      };
      if (arg == "--scene_dir" || arg == "--scene-dir") {
        scene_dir = value(arg.c_str());
      } else if (arg == "--dem") {
        dem_path = value(arg.c_str());
      } else if (arg == "--albedo") {
        albedo_path = value(arg.c_str());
      } else if (arg == "--traj") {
        traj_path = value(arg.c_str());
      } else if (arg == "--output") {
        output_dir = value(arg.c_str());
      } else if (arg == "--config") {
        config_path = value(arg.c_str());
      } else if (arg == "--event_format" || arg == "--event-format" || arg == "--events_format" ||
                 arg == "--events-format") {
        event_format = value(arg.c_str());
        if (event_format == "h5") event_format = "hdf5";
        else if (event_format == "binary") event_format = "bin";
        if (event_format != "bin" && event_format != "hdf5")
          throw std::runtime_error("invalid event format for --event_format: " + event_format +
                                   " (expected bin or hdf5)");
      } else if (arg == "--solver") {
        event_solver = value(arg.c_str());
        if (event_solver != "auto" && event_solver != "native" && event_solver != "adaptive-optics")
          throw std::runtime_error("solver must be auto, native, or adaptive-optics");
      } else if (arg == "--bvh") {
        bvh = value(arg.c_str());
        if (bvh != "fp32" && bvh != "half" && bvh != "watertight" && bvh != "half+watertight")
          throw std::runtime_error("bvh must be fp32, half, watertight, or half+watertight");
      } else if (arg == "--circuit") {
        circuit = value(arg.c_str());
        if (circuit != "fp64" && circuit != "fp32" && circuit != "fp32-philox")
          throw std::runtime_error("circuit must be fp64, fp32, or fp32-philox");
      } else if (arg == "--help" || arg == "-h") {
        print_usage(argv[0]);
        std::exit(0);
      } else {
        throw std::runtime_error("unknown argument: " + arg);
      }
    }
    if (scene_dir.empty() && (dem_path.empty() || traj_path.empty()))
      throw std::runtime_error("either --scene_dir or --dem and --traj are required");
    std::ifstream config_in(config_path);
    if (!config_in.good()) throw std::runtime_error("failed to open config file: " + config_path);
  }
};

}  // namespace dvs_app
