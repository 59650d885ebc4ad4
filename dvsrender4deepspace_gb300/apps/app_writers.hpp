// Output formats of the drop-in apps.
//
// * events.bin -- the reference's legacy 13-byte records
//   {float32 t, int16 x, int16 y, int8 p, float32 depth} (dvs_writer.hpp:44-55).
// * events.h5  -- datasets x (int16), y (int16), t (int64 microseconds),
//   p (int8) and ms_to_idx (int64: index of the first event at or after each
//   millisecond) with the reference's ordering, rounding and bound checks
//   (dvs_writer.hpp:70-264).  No HDF5 library is available, so the file is
//   written directly in the HDF5 file format (version 0 superblock, one
//   root group with a symbol table, contiguous one-dimensional datasets);
//   the columns are spooled to side files while events are appended and
//   assembled at close.
// * PNG (8-bit grey, stored deflate blocks) and float32 TIFF (uncompressed),
//   the image and depth files of bin/cam, with the reference's preview
//   encoding (blenderize.hpp:12-69).
#pragma once
#include <cstdint>
#include <fstream>
#include <string>
#include <vector>

#include "dvs_gb300.h"

namespace dvs_app {

class EventStreamWriter {
 public:
  virtual ~EventStreamWriter() = default;
  virtual void append(std::vector<dvs_event> events) = 0;
  virtual void close(double end_time_seconds) = 0;
  virtual const std::string &path() const = 0;
  size_t event_count() const { return event_count_; }

 protected:
  size_t event_count_ = 0;
};

class BinaryEventStreamWriter final : public EventStreamWriter {
 public:
  explicit BinaryEventStreamWriter(std::string path);
  void append(std::vector<dvs_event> events) override;
  void close(double) override { out_.close(); }
  const std::string &path() const override { return path_; }

 private:
  std::string path_;
  std::ofstream out_;
};

class Hdf5EventStreamWriter final : public EventStreamWriter {
 public:
  explicit Hdf5EventStreamWriter(std::string path);
  ~Hdf5EventStreamWriter() override;
  void append(std::vector<dvs_event> events) override;
  void close(double end_time_seconds) override;
  const std::string &path() const override { return path_; }

 private:
  void fill_ms_to_idx(int64_t target_ms, size_t event_index);
  std::string path_;
  std::ofstream col_[4];  // x, y, t, p spool files
  std::vector<int64_t> ms_to_idx_;
  int64_t last_ms_ = -1;
  double last_timestamp_;
  bool closed_ = false;
};

// One named, contiguous, one-dimensional integer dataset of an HDF5 file.
struct Hdf5Column {
  std::string name;
  int element_size;          // bytes: 1, 2, 4 or 8 (signed little-endian integers)
  uint64_t count;            // elements
  std::string source_file;   // raw little-endian data (count * element_size bytes), or empty
  const void *data = nullptr;  // used when source_file is empty
};
// Writes an HDF5 file holding the columns in the root group.
void write_hdf5_columns(const std::string &path, std::vector<Hdf5Column> columns);

// Preview encoding of a linear radiance image (blenderize.hpp:12-69).
uint8_t to_byte(float v);
float linear_to_srgb(float c);
float display_exposure(float x);
void render_float_to_png_bytes(const float *linear, int width, int height, float dither, std::vector<uint8_t> &out);
void write_png_gray8(const std::string &path, const uint8_t *pixels, int width, int height);
void write_tiff_float32(const std::string &path, const float *pixels, int width, int height);

}  // namespace dvs_app
