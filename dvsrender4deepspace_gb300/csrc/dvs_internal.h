// Internal data layout of the GB300 DVS path, shared by host C++ and device
// code.  Nothing here is part of the C-ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "dvs_gb300.h"

namespace dvsgb {

// ---- wide BVH --------------------------------------------------------------
// An 8-wide node is eight 32-byte child records (256 bytes).  Lane c of a
// warp reads child record c with two 16-byte loads, so the eight lanes that
// test one node read it as one coalesced 256-byte access.
// child: inner node index when count==0, first triangle (leaf order) when
// count>0; count<0 marks an empty slot.
constexpr int kBvhWidth = 8;
struct alignas(32) BvhChild {
  float lo[3];
  float hi[3];
  int32_t child;
  int32_t count;
};
struct alignas(256) BvhNode {
  BvhChild c[kBvhWidth];
};
static_assert(sizeof(BvhChild) == 32, "BvhChild layout");
static_assert(sizeof(BvhNode) == 256, "BvhNode layout");

// Precision-format node (FP16 child bounds), 144 bytes: a 16-byte header with
// the node's FP32 origin (the minimum corner of its children) and eight
// 16-byte children.  A child's bounds are FP16 offsets from the origin, lower
// bounds rounded toward -inf and upper bounds toward +inf; the device adds
// them to the origin with the same directed rounding (__fadd_rd/__fadd_ru),
// so a decoded box always encloses the FP32 box.  link: inner child = node
// index (bit 31 clear); leaf = bit 31 | (triangles - 1) << 27 | first
// triangle (27 bits); empty slot = all ones.
struct alignas(16) BvhQChild {
  uint16_t lo[3];
  uint16_t hi[3];
  uint32_t link;
};
struct alignas(16) BvhQNode {
  float origin[3];
  uint32_t pad;
  BvhQChild c[kBvhWidth];
};
static_assert(sizeof(BvhQChild) == 16, "BvhQChild layout");
static_assert(sizeof(BvhQNode) == 144, "BvhQNode layout");
constexpr uint32_t kQLinkEmpty = 0xffffffffu;
constexpr uint32_t kQLinkLeaf = 0x80000000u;
constexpr uint32_t kQLinkFirstMask = 0x07ffffffu;
constexpr int kQLinkCountShift = 27;

// Intersection record in leaf order, 48 bytes = 3 x 16-byte loads.  Edges are
// precomputed with the same float subtraction the reference performs per test
// (include/dvs/device_ray.hpp:58-59), so the Moller-Trumbore inputs are
// bit-identical.  Precision scenes store the vertices instead (v0, v1, v2 in
// the v0/e1/e2 slots) for the watertight test.
struct alignas(16) TriRecord {
  float v0[3];
  float e1[3];
  float e2[3];
  uint32_t original;  // triangle index in the caller's mesh
  uint32_t pad[2];
};
static_assert(sizeof(TriRecord) == 48, "TriRecord layout");

// Shading record in leaf order, 64 bytes: vertex normals and per-vertex
// material albedo (already passed through the fallback rule of
// include/dvs/device_optics.cuh:30-33).
struct alignas(16) ShadeRecord {
  float n0[3], a0;
  float n1[3], a1;
  float n2[3], a2;
  float pad[4];
};
static_assert(sizeof(ShadeRecord) == 64, "ShadeRecord layout");

// Maximum warp-stack depth; the builder rejects trees that could exceed it
// (a depth-first walk of a W-wide tree holds at most (W-1)*depth+1 entries).
constexpr int kStackSlots = 96;

struct BvhBuild {
  std::vector<BvhNode> nodes;
  std::vector<uint32_t> order;  // leaf order -> original triangle index
  int depth = 0;                // levels of wide nodes
  double seconds = 0;
  // surface-area model of the wide tree: expected wide nodes visited and
  // triangle tests of a ray through the root box
  double sah_node_visits = 0, sah_triangle_tests = 0;
};

// Binary tree collapsed to an 8-wide tree; builder 0 splits by binned SAH,
// builder 1 splits Morton-ordered ranges at their highest differing code bit.
// collapse 1 (the default) chooses the wide nodes by surface-area cost over
// slot budgets, collapse 0 opens the largest-area child greedily.  Returns
// false with a message on invalid input.
bool build_bvh(const float *vertices, size_t n_vertices, const uint32_t *indices, size_t n_triangles,
               int leaf_size, int builder, BvhBuild &out, std::string &error, int collapse = 1);

// The precision-format copy of a built tree (same node indices).  Fails when a
// leaf's first triangle or size does not fit the link, or when a decoded box
// would not enclose its FP32 box (checked for every child).
bool quantize_bvh(const std::vector<BvhNode> &nodes, std::vector<BvhQNode> &out, std::string &error);

// ---- FIFO readout (src/event_readout.cpp:6-34 semantics) ---------------------
struct HostEvent {
  double t;
  int16_t x, y;
  int8_t p;
  float depth;
};

class Readout {
 public:
  Readout(double bandwidth, double latency, size_t capacity)
      : bandwidth_(bandwidth), latency_(latency), capacity_(capacity) {}
  // Orders a batch by (t, y, x), queues it and appends the events whose
  // delivery time is <= now to `ready`.
  void submit(std::vector<HostEvent> &batch, double now, std::vector<HostEvent> &ready);
  void drain(std::vector<HostEvent> &ready);
  size_t dropped() const { return dropped_; }
  size_t peak() const { return peak_; }

 private:
  struct Pending {
    double ready_time;
    HostEvent event;
  };
  double bandwidth_, latency_, available_ = 0;
  size_t capacity_, dropped_ = 0, peak_ = 0;
  std::vector<Pending> queue_;
  size_t head_ = 0;
};

}  // namespace dvsgb
