// Driver for the host-side tests of the apps' writers (tests/test_apps_host.py):
// writes files the Python side reads back with independent readers.
//   apps_selftest events <dir>   events.bin / events.h5 of tests/test_writer.cpp:11-18,
//                                an empty events.h5 and the writer's refusals
//   apps_selftest images <dir>   preview PNG and float32 TIFF of a known image
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "app_writers.hpp"

using namespace dvs_app;

static dvs_event ev(double t, int x, int y, int p, float depth) {
  dvs_event e{};
  e.timestamp = t;
  e.x = int16_t(x);
  e.y = int16_t(y);
  e.polarity = int8_t(p);
  e.depth = depth;
  return e;
}

template <typename F>
static void expect_error(const char *what, F f) {
  try {
    f();
  } catch (const std::exception &e) {
    std::cout << "refused " << what << ": " << e.what() << "\n";
    return;
  }
  std::cout << "accepted " << what << "\n";
}

int main(int argc, char **argv) {
  try {
    if (argc < 3) throw std::invalid_argument("usage: apps_selftest events|images <dir>");
    const std::string mode = argv[1], dir = argv[2];
    std::filesystem::create_directories(dir);
    if (mode == "events") {
      {
        BinaryEventStreamWriter w(dir + "/events.bin");
        w.append({ev(.001234, 2, 3, 1, 10), ev(.0021, 4, 5, 0, 20)});
        w.close(.003);
      }
      {
        Hdf5EventStreamWriter w(dir + "/events.h5");
        w.append({ev(.0021, 4, 5, 0, 20), ev(.001234, 2, 3, 1, 10)});  // sorted on append
        w.append({ev(50.000001, 2, 3, 1, 10), ev(50.000002, 2, 3, 1, 10)});
        w.close(50.001);
        std::cout << "h5 events " << w.event_count() << "\n";
      }
      {
        Hdf5EventStreamWriter w(dir + "/empty.h5");
        w.close(-1);
      }
      expect_error("unordered batches", [&] {
        Hdf5EventStreamWriter w(dir + "/bad.h5");
        w.append({ev(1.0, 0, 0, 1, 1)});
        w.append({ev(0.5, 0, 0, 1, 1)});
      });
      expect_error("negative timestamp", [&] {
        Hdf5EventStreamWriter w(dir + "/bad.h5");
        w.append({ev(-1e-3, 0, 0, 1, 1)});
      });
      expect_error("append after close", [&] {
        Hdf5EventStreamWriter w(dir + "/bad.h5");
        w.close(0.0);
        w.append({ev(1.0, 0, 0, 1, 1)});
      });
      expect_error("nonfinite end", [&] {
        Hdf5EventStreamWriter w(dir + "/bad.h5");
        w.close(std::nan(""));
      });
    } else if (mode == "images") {
      const int w = 37, h = 5;
      std::vector<float> img(size_t(w) * h), depth(size_t(w) * h);
      for (int i = 0; i < w * h; ++i) {
        img[size_t(i)] = float(i) * 0.7f;       // 0 .. 128: through the exposure clamp
        depth[size_t(i)] = i % 7 == 0 ? -1.0f : 100.0f + 0.25f * float(i);
      }
      std::vector<uint8_t> bytes;
      render_float_to_png_bytes(img.data(), w, h, 0.0f, bytes);
      write_png_gray8(dir + "/image.png", bytes.data(), w, h);
      write_tiff_float32(dir + "/depth.tif", depth.data(), w, h);
      // a PNG larger than one stored deflate block
      const int W = 300, H = 260;
      std::vector<uint8_t> big(size_t(W) * H);
      for (size_t i = 0; i < big.size(); ++i) big[i] = uint8_t((i * 7) & 0xff);
      write_png_gray8(dir + "/big.png", big.data(), W, H);
      std::cout << "encoded";
      for (uint8_t b : bytes) std::cout << " " << int(b);
      std::cout << "\n";
    } else {
      throw std::invalid_argument("unknown mode " + mode);
    }
    return 0;
  } catch (const std::exception &e) {
    std::cerr << "FAIL: " << e.what() << "\n";
    return 1;
  }
}
