// Output formats of the drop-in apps: events.bin, events.h5, PNG and TIFF.
#include "app_writers.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>

namespace dvs_app {

// ---- events.bin ------------------------------------------------------------------
BinaryEventStreamWriter::BinaryEventStreamWriter(std::string path) : path_(std::move(path)) {
  out_.open(path_, std::ios::binary);
  if (!out_) throw std::runtime_error("failed to open output file: " + path_);
}

void BinaryEventStreamWriter::append(std::vector<dvs_event> events) {
  if (events.empty()) return;
#pragma pack(push, 1)
  struct Record {
    float t;
    int16_t x, y;
    int8_t p;
    float depth;
  };
#pragma pack(pop)
  static_assert(sizeof(Record) == 13, "legacy 13-byte event record");
  std::vector<Record> rec(events.size());
  for (size_t i = 0; i < events.size(); ++i)
    rec[i] = Record{float(events[i].timestamp), events[i].x, events[i].y, events[i].polarity, events[i].depth};
  out_.write(reinterpret_cast<const char *>(rec.data()), std::streamsize(rec.size() * sizeof(Record)));
  out_.flush();
  if (!out_) throw std::runtime_error("failed to write output file: " + path_);
  event_count_ += events.size();
}

// ---- events.h5 -------------------------------------------------------------------
static const char *kColumnNames[4] = {"x", "y", "t", "p"};

Hdf5EventStreamWriter::Hdf5EventStreamWriter(std::string path)
    : path_(std::move(path)), last_timestamp_(-std::numeric_limits<double>::infinity()) {
  // the output must be creatable now, as with H5Fcreate
  std::ofstream probe(path_, std::ios::binary | std::ios::trunc);
  if (!probe) throw std::runtime_error("failed to create HDF5 file: " + path_);
  for (int c = 0; c < 4; ++c) {
    col_[c].open(path_ + "." + kColumnNames[c] + ".spool", std::ios::binary | std::ios::trunc);
    if (!col_[c]) throw std::runtime_error("failed to create HDF5 file: " + path_);
  }
}

Hdf5EventStreamWriter::~Hdf5EventStreamWriter() {
  for (int c = 0; c < 4; ++c) {
    if (col_[c].is_open()) col_[c].close();
    std::remove((path_ + "." + kColumnNames[c] + ".spool").c_str());
  }
}

void Hdf5EventStreamWriter::fill_ms_to_idx(int64_t target_ms, size_t event_index) {
  if (target_ms < 0) return;
  if (target_ms > int64_t(std::numeric_limits<int>::max()))
    throw std::runtime_error("ms_to_idx would be unreasonably large");
  while (last_ms_ < target_ms) {
    ms_to_idx_.push_back(int64_t(event_index));
    ++last_ms_;
  }
}

void Hdf5EventStreamWriter::append(std::vector<dvs_event> events) {
  if (closed_) throw std::runtime_error("cannot append to closed HDF5 event file");
  if (events.empty()) return;
  for (const dvs_event &e : events)
    if (!std::isfinite(e.timestamp) || e.timestamp < 0 || e.timestamp * 1000 > std::numeric_limits<int>::max() - 1)
      throw std::runtime_error("HDF5 event timestamp is outside millisecond-index bounds");
  std::stable_sort(events.begin(), events.end(),
                   [](const dvs_event &a, const dvs_event &b) { return a.timestamp < b.timestamp; });
  if (events.front().timestamp < last_timestamp_) throw std::runtime_error("HDF5 events must be globally time ordered");
  const size_t n = events.size();
  std::vector<int16_t> xs(n), ys(n);
  std::vector<int64_t> ts(n);
  std::vector<int8_t> ps(n);
  for (size_t i = 0; i < n; ++i) {
    xs[i] = events[i].x;
    ys[i] = events[i].y;
    ts[i] = std::llround(events[i].timestamp * 1e6);  // microseconds
    ps[i] = events[i].polarity;
  }
  col_[0].write(reinterpret_cast<const char *>(xs.data()), std::streamsize(n * 2));
  col_[1].write(reinterpret_cast<const char *>(ys.data()), std::streamsize(n * 2));
  col_[2].write(reinterpret_cast<const char *>(ts.data()), std::streamsize(n * 8));
  col_[3].write(reinterpret_cast<const char *>(ps.data()), std::streamsize(n));
  for (int c = 0; c < 4; ++c)
    if (!col_[c]) throw std::runtime_error("failed to write HDF5 event dataset");
  for (size_t i = 0; i < n; ++i) fill_ms_to_idx(ts[i] / 1000, event_count_ + i);
  last_timestamp_ = events.back().timestamp;
  event_count_ += n;
}

void Hdf5EventStreamWriter::close(double end_ts_s) {
  if (closed_) return;
  if (!std::isfinite(end_ts_s) || end_ts_s * 1000 > std::numeric_limits<int>::max() - 1)
    throw std::runtime_error("invalid HDF5 observation end time");
  const int64_t end_ms = end_ts_s < 0 ? -1 : std::llround(end_ts_s * 1000);
  if (end_ms >= 0) fill_ms_to_idx(end_ms, event_count_);
  for (int c = 0; c < 4; ++c) col_[c].close();
  std::vector<Hdf5Column> cols;
  const int sizes[4] = {2, 2, 8, 1};
  for (int c = 0; c < 4; ++c)
    cols.push_back(Hdf5Column{kColumnNames[c], sizes[c], event_count_, path_ + "." + kColumnNames[c] + ".spool"});
  Hdf5Column idx{"ms_to_idx", 8, ms_to_idx_.size(), std::string()};
  idx.data = ms_to_idx_.data();
  cols.push_back(idx);
  write_hdf5_columns(path_, cols);
  for (int c = 0; c < 4; ++c) std::remove((path_ + "." + kColumnNames[c] + ".spool").c_str());
  closed_ = true;
}

// ---- HDF5 file format (version 0 superblock, v1 object headers) -------------------
namespace {

constexpr uint64_t kUndef = ~uint64_t(0);

struct Bytes {
  std::vector<uint8_t> b;
  void u8(uint64_t v) { b.push_back(uint8_t(v)); }
  void u16(uint64_t v) { for (int i = 0; i < 2; ++i) b.push_back(uint8_t(v >> (8 * i))); }
  void u32(uint64_t v) { for (int i = 0; i < 4; ++i) b.push_back(uint8_t(v >> (8 * i))); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back(uint8_t(v >> (8 * i))); }
  void raw(const char *s, size_t n) { b.insert(b.end(), s, s + n); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
  size_t size() const { return b.size(); }
};

// One object header message: type, data (padded to 8 bytes).
void message(Bytes &out, int type, const Bytes &data) {
  Bytes d = data;
  d.pad8();
  out.u16(uint64_t(type));
  out.u16(d.size());
  out.u8(0);      // flags
  out.zeros(3);   // reserved
  out.b.insert(out.b.end(), d.b.begin(), d.b.end());
}

// Version 1 object header around the given messages.
Bytes object_header(const std::vector<Bytes> &messages_with_headers, int count) {
  size_t body = 0;
  for (const Bytes &m : messages_with_headers) body += m.size();
  Bytes h;
  h.u8(1);       // version
  h.u8(0);       // reserved
  h.u16(uint64_t(count));
  h.u32(1);      // reference count
  h.u32(body);   // header data size
  h.zeros(4);    // alignment of the first message to 8 bytes
  for (const Bytes &m : messages_with_headers) h.b.insert(h.b.end(), m.b.begin(), m.b.end());
  return h;
}

Bytes dataset_header(uint64_t count, int element_size, uint64_t data_address) {
  std::vector<Bytes> msgs(4);
  Bytes space;  // dataspace, version 1: rank 1, no maximum dimensions
  space.u8(1);
  space.u8(1);
  space.u8(0);
  space.zeros(5);
  space.u64(count);
  message(msgs[0], 0x0001, space);
  Bytes type;  // datatype, version 1, fixed-point, little-endian, signed
  type.u8(0x10);
  type.u8(0x08);
  type.u8(0);
  type.u8(0);
  type.u32(uint64_t(element_size));
  type.u16(0);                          // bit offset
  type.u16(uint64_t(element_size) * 8);  // bit precision
  message(msgs[1], 0x0003, type);
  Bytes fill;  // fill value, version 2: allocation late, write if set, undefined
  fill.u8(2);
  fill.u8(2);
  fill.u8(2);
  fill.u8(0);
  message(msgs[2], 0x0005, fill);
  Bytes layout;  // data layout, version 3, contiguous
  layout.u8(3);
  layout.u8(1);
  layout.u64(count ? data_address : kUndef);
  layout.u64(count * uint64_t(element_size));
  message(msgs[3], 0x0008, layout);
  return object_header(msgs, 4);
}

void copy_file_into(std::ofstream &out, const std::string &src, uint64_t bytes) {
  std::ifstream in(src, std::ios::binary);
  if (!in) throw std::runtime_error("failed to read HDF5 spool file: " + src);
  std::vector<char> buf(1 << 22);
  uint64_t left = bytes;
  while (left) {
    const std::streamsize n = std::streamsize(std::min<uint64_t>(left, buf.size()));
    in.read(buf.data(), n);
    if (in.gcount() != n) throw std::runtime_error("short HDF5 spool file: " + src);
    out.write(buf.data(), n);
    left -= uint64_t(n);
  }
}

}  // namespace

void write_hdf5_columns(const std::string &path, std::vector<Hdf5Column> cols) {
  // symbol table entries are looked up by binary search: sort by name
  std::sort(cols.begin(), cols.end(), [](const Hdf5Column &a, const Hdf5Column &b) { return a.name < b.name; });
  const int leaf_k = 4, internal_k = 16;
  if (cols.size() > size_t(2 * leaf_k)) throw std::invalid_argument("too many HDF5 columns for one symbol node");

  // local heap data: "" at 0, then each name, 8-byte aligned
  Bytes heap_data;
  heap_data.zeros(8);
  std::vector<uint64_t> name_off;
  for (const Hdf5Column &c : cols) {
    name_off.push_back(heap_data.size());
    heap_data.raw(c.name.c_str(), c.name.size() + 1);
    heap_data.pad8();
  }

  const uint64_t a_super = 0, super_size = 96;
  const uint64_t a_root = a_super + super_size, root_size = 16 + 8 + 16;
  const uint64_t a_heap = a_root + root_size, heap_hdr = 32;
  const uint64_t a_heap_data = a_heap + heap_hdr;
  const uint64_t a_btree = a_heap_data + heap_data.size();
  const uint64_t btree_size = 24 + uint64_t(2 * internal_k) * 8 + uint64_t(2 * internal_k + 1) * 8;
  const uint64_t a_snod = a_btree + btree_size, snod_size = 8 + uint64_t(2 * leaf_k) * 40;
  const uint64_t a_ds = a_snod + snod_size, ds_size = 16 + 24 + 24 + 16 + 32;
  uint64_t a_data = a_ds + ds_size * cols.size();
  a_data = (a_data + 63) & ~uint64_t(63);
  std::vector<uint64_t> data_addr;
  uint64_t eof = a_data;
  for (const Hdf5Column &c : cols) {
    data_addr.push_back(eof);
    eof += c.count * uint64_t(c.element_size);
  }

  Bytes meta;
  // superblock
  meta.raw("\x89HDF\r\n\x1a\n", 8);
  meta.u8(0);  // superblock version
  meta.u8(0);  // free-space version
  meta.u8(0);  // root group symbol table entry version
  meta.u8(0);
  meta.u8(0);  // shared header message format version
  meta.u8(8);  // size of offsets
  meta.u8(8);  // size of lengths
  meta.u8(0);
  meta.u16(uint64_t(leaf_k));
  meta.u16(uint64_t(internal_k));
  meta.u32(0);  // file consistency flags
  meta.u64(0);  // base address
  meta.u64(kUndef);  // free-space info
  meta.u64(eof);     // end of file
  meta.u64(kUndef);  // driver info
  // root group symbol table entry: cached B-tree and heap addresses
  meta.u64(0);
  meta.u64(a_root);
  meta.u32(1);
  meta.u32(0);
  meta.u64(a_btree);
  meta.u64(a_heap);
  // root group object header: one symbol table message
  {
    std::vector<Bytes> msgs(1);
    Bytes st;
    st.u64(a_btree);
    st.u64(a_heap);
    message(msgs[0], 0x0011, st);
    const Bytes oh = object_header(msgs, 1);
    meta.b.insert(meta.b.end(), oh.b.begin(), oh.b.end());
  }
  // local heap (no free blocks: free-list head = 1, the format's null offset)
  meta.raw("HEAP", 4);
  meta.u8(0);
  meta.zeros(3);
  meta.u64(heap_data.size());
  meta.u64(1);
  meta.u64(a_heap_data);
  meta.b.insert(meta.b.end(), heap_data.b.begin(), heap_data.b.end());
  // group B-tree: one leaf node pointing at one symbol table node
  {
    const size_t start = meta.size();
    meta.raw("TREE", 4);
    meta.u8(0);  // group node
    meta.u8(0);  // leaf level
    meta.u16(1);
    meta.u64(kUndef);
    meta.u64(kUndef);
    meta.u64(0);                 // key 0: "" (below every name)
    meta.u64(a_snod);            // child 0
    meta.u64(name_off.empty() ? 0 : name_off.back());  // key 1: the largest name
    meta.zeros(btree_size - (meta.size() - start));
  }
  // symbol table node
  {
    const size_t start = meta.size();
    meta.raw("SNOD", 4);
    meta.u8(1);
    meta.u8(0);
    meta.u16(cols.size());
    for (size_t i = 0; i < cols.size(); ++i) {
      meta.u64(name_off[i]);
      meta.u64(a_ds + ds_size * i);
      meta.u32(0);
      meta.u32(0);
      meta.zeros(16);
    }
    meta.zeros(snod_size - (meta.size() - start));
  }
  for (size_t i = 0; i < cols.size(); ++i) {
    const Bytes oh = dataset_header(cols[i].count, cols[i].element_size, data_addr[i]);
    if (oh.size() != ds_size) throw std::logic_error("HDF5 dataset header size");
    meta.b.insert(meta.b.end(), oh.b.begin(), oh.b.end());
  }
  meta.zeros(a_data - meta.size());

  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) throw std::runtime_error("failed to create HDF5 file: " + path);
  out.write(reinterpret_cast<const char *>(meta.b.data()), std::streamsize(meta.size()));
  for (const Hdf5Column &c : cols) {
    const uint64_t bytes = c.count * uint64_t(c.element_size);
    if (!bytes) continue;
    if (!c.source_file.empty()) copy_file_into(out, c.source_file, bytes);
    else out.write(static_cast<const char *>(c.data), std::streamsize(bytes));
  }
  out.flush();
  if (!out) throw std::runtime_error("failed to close event file");
}

// ---- preview images --------------------------------------------------------------
uint8_t to_byte(float v) {
  if (!std::isfinite(v) || v <= 0.0f) return 0;
  if (v >= 1.0f) return 255;
  return uint8_t(v * 255.0f + 0.5f);
}

float linear_to_srgb(float c) {
  if (c < 0.0031308f) return 12.92f * c;
  return 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f;
}

float display_exposure(float x) { return std::clamp(x / 100, 0.0f, 1.0f); }

// Integer hash dither with a triangular distribution (Blender's preview path).
static float random_dither(int x, int y) {
  const uint32_t ux = uint32_t(x), uy = uint32_t(y);
  const uint32_t qx = 1103515245u * ((ux >> 1u) ^ uy);
  const uint32_t qy = 1103515245u * ((uy >> 1u) ^ ux);
  const uint32_t n = 1103515245u * (qx ^ (qy >> 3u));
  float v = float(n) * (1.0f / float(0xffffffffu));
  v = v * 2.0f - 1.0f;
  return std::copysign(1.0f, v) * (1.0f - std::sqrt(1.0f - std::fabs(v)));
}

void render_float_to_png_bytes(const float *linear, int width, int height, float dither, std::vector<uint8_t> &out) {
  out.resize(size_t(width) * height);
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      float r = linear_to_srgb(display_exposure(linear[size_t(y) * width + x]));
      r += dither * random_dither(x, y);
      out[size_t(y) * width + x] = to_byte(r);
    }
}

namespace {

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    ready = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

void be32(std::vector<uint8_t> &v, uint32_t x) {
  for (int i = 3; i >= 0; --i) v.push_back(uint8_t(x >> (8 * i)));
}

void png_chunk(std::ofstream &out, const char type[4], const std::vector<uint8_t> &data) {
  std::vector<uint8_t> head;
  be32(head, uint32_t(data.size()));
  out.write(reinterpret_cast<const char *>(head.data()), 4);
  std::vector<uint8_t> body(type, type + 4);
  body.insert(body.end(), data.begin(), data.end());
  out.write(reinterpret_cast<const char *>(body.data()), std::streamsize(body.size()));
  std::vector<uint8_t> crc;
  be32(crc, crc32_update(0, body.data(), body.size()));
  out.write(reinterpret_cast<const char *>(crc.data()), 4);
}

}  // namespace

void write_png_gray8(const std::string &path, const uint8_t *pixels, int width, int height) {
  if (width <= 0 || height <= 0) throw std::invalid_argument("invalid PNG size");
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) throw std::runtime_error("failed to open output file: " + path);
  out.write("\x89PNG\r\n\x1a\n", 8);
  std::vector<uint8_t> ihdr;
  be32(ihdr, uint32_t(width));
  be32(ihdr, uint32_t(height));
  ihdr.insert(ihdr.end(), {8, 0, 0, 0, 0});  // 8-bit grey, deflate, no filter, no interlace
  png_chunk(out, "IHDR", ihdr);
  // scanlines with filter byte 0, in a zlib stream of stored deflate blocks
  std::vector<uint8_t> raw;
  raw.reserve(size_t(height) * (size_t(width) + 1));
  for (int y = 0; y < height; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), pixels + size_t(y) * width, pixels + size_t(y + 1) * width);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  size_t pos = 0;
  do {
    const size_t n = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + n == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back(uint8_t(n));
    z.push_back(uint8_t(n >> 8));
    z.push_back(uint8_t(~n));
    z.push_back(uint8_t(~n >> 8));
    z.insert(z.end(), raw.begin() + long(pos), raw.begin() + long(pos + n));
    pos += n;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  be32(z, (b << 16) | a);
  png_chunk(out, "IDAT", z);
  png_chunk(out, "IEND", {});
  if (!out) throw std::runtime_error("failed to write output file: " + path);
}

void write_tiff_float32(const std::string &path, const float *pixels, int width, int height) {
  if (width <= 0 || height <= 0) throw std::invalid_argument("invalid TIFF size");
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) throw std::runtime_error("failed to open output file: " + path);
  const uint32_t bytes = uint32_t(width) * uint32_t(height) * 4u;
  Bytes h;
  h.raw("II", 2);
  h.u16(42);
  h.u32(8 + bytes + (bytes & 1));  // IFD after the pixels
  out.write(reinterpret_cast<const char *>(h.b.data()), std::streamsize(h.size()));
  out.write(reinterpret_cast<const char *>(pixels), bytes);  // host is little-endian (x86-64, aarch64)
  if (bytes & 1) out.put(0);
  struct Tag {
    uint16_t tag, type;
    uint32_t value;
  };
  const Tag tags[] = {{256, 4, uint32_t(width)}, {257, 4, uint32_t(height)}, {258, 3, 32}, {259, 3, 1},
                      {262, 3, 1}, {273, 4, 8}, {277, 3, 1}, {278, 4, uint32_t(height)}, {279, 4, bytes},
                      {284, 3, 1}, {339, 3, 3}};
  Bytes ifd;
  ifd.u16(sizeof(tags) / sizeof(tags[0]));
  for (const Tag &t : tags) {
    ifd.u16(t.tag);
    ifd.u16(t.type);
    ifd.u32(1);
    if (t.type == 3) {  // SHORT: left-justified in the value field
      ifd.u16(t.value);
      ifd.u16(0);
    } else {
      ifd.u32(t.value);
    }
  }
  ifd.u32(0);
  out.write(reinterpret_cast<const char *>(ifd.b.data()), std::streamsize(ifd.size()));
  if (!out) throw std::runtime_error("failed to write output file: " + path);
}

}  // namespace dvs_app
