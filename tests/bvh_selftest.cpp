// Host-side check of the wide-BVH builder and of the FP16 child-bound
// quantisation (tests/test_bvh_host.py), linked against libdvs_gb300.so.
//   bvh_selftest <seed> <n> <scale>   a jittered n x n grid mesh at coordinates
//                                     up to `scale`, built with leaf 2 and quantised
// Prints "nodes <n> depth <d> leaves <l> max_slack <s>" and exits 0 when
//   * every triangle appears in exactly one leaf, and every child box encloses
//     the boxes (or triangles) below it;
//   * every quantised child decodes (origin + offset, rounded toward -inf for
//     lower and +inf for upper bounds, as the device does) to a box that
//     encloses its FP32 box, with the same link (inner node, leaf range, empty);
// max_slack: the largest widening of a decoded box relative to its node's extent.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "dvs_internal.h"

using namespace dvsgb;

static double half_value(uint16_t h) {
  const int E = (h >> 10) & 31, m = h & 1023;
  if (E == 31) return m ? NAN : INFINITY;
  return E == 0 ? std::ldexp((double)m, -24) : std::ldexp((double)(1024 + m), E - 25);
}
// origin + offset rounded to float toward -inf (up = false) or +inf, through
// the floating-point environment's directed rounding (an independent route
// from the library's own check)
static float add_rounded(float origin, uint16_t off, bool up) {
  const float h = (float)half_value(off);  // exact: every half is a float
  const int old = std::fegetround();
  std::fesetround(up ? FE_UPWARD : FE_DOWNWARD);
  volatile float a = origin, b = h;
  volatile float r = a + b;
  std::fesetround(old);
  return r;
}

int main(int argc, char **argv) {
  if (argc < 4 || argc > 6) return 2;
  const unsigned seed = (unsigned)std::atoi(argv[1]);
  const int n = std::atoi(argv[2]);
  const double scale = std::atof(argv[3]);
  const int builder = argc >= 5 ? std::atoi(argv[4]) : 0;   // 0 binned SAH, 1 Morton radix
  const int collapse = argc == 6 ? std::atoi(argv[5]) : 1;  // 1 slot budgets (default), 0 greedy
  std::mt19937 rng(seed);
  std::uniform_real_distribution<double> jitter(-0.3, 0.3), height(0.0, 1.0);
  std::vector<float> V;
  const double step = scale / n;
  for (int y = 0; y < n; ++y)
    for (int x = 0; x < n; ++x) {
      V.push_back((float)((x + jitter(rng)) * step - scale / 2));
      V.push_back((float)((y + jitter(rng)) * step - scale / 2));
      V.push_back((float)(height(rng) * step * 3));
    }
  std::vector<uint32_t> I;
  for (int y = 0; y + 1 < n; ++y)
    for (int x = 0; x + 1 < n; ++x) {
      const uint32_t a = y * n + x, b = a + 1, c = a + n, d = c + 1;
      I.insert(I.end(), {a, b, d, a, d, c});
    }
  const size_t nt = I.size() / 3;
  BvhBuild bvh;
  std::string err;
  if (!build_bvh(V.data(), V.size() / 3, I.data(), nt, 2, builder, bvh, err, collapse)) {
    std::printf("build failed: %s\n", err.c_str());
    return 1;
  }
  std::vector<BvhQNode> q;
  if (!quantize_bvh(bvh.nodes, q, err)) {
    std::printf("quantize failed: %s\n", err.c_str());
    return 1;
  }
  // leaves cover every triangle once; child boxes enclose their triangles
  std::vector<int> seen(nt, 0);
  size_t leaves = 0;
  double max_slack = 0;
  for (size_t i = 0; i < bvh.nodes.size(); ++i) {
    const BvhNode &node = bvh.nodes[i];
    const BvhQNode &qn = q[i];
    float lo_n[3] = {INFINITY, INFINITY, INFINITY}, hi_n[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < kBvhWidth; ++k)
      if (node.c[k].count >= 0)
        for (int d = 0; d < 3; ++d) {
          lo_n[d] = std::fmin(lo_n[d], node.c[k].lo[d]);
          hi_n[d] = std::fmax(hi_n[d], node.c[k].hi[d]);
        }
    for (int k = 0; k < kBvhWidth; ++k) {
      const BvhChild &c = node.c[k];
      const BvhQChild &qc = qn.c[k];
      if (c.count < 0) {
        if (qc.link != kQLinkEmpty) { std::printf("empty link %zu/%d\n", i, k); return 1; }
        continue;
      }
      if (c.count == 0) {
        if (qc.link != (uint32_t)c.child) { std::printf("inner link %zu/%d\n", i, k); return 1; }
      } else {
        const uint32_t want = kQLinkLeaf | ((uint32_t)(c.count - 1) << kQLinkCountShift) | (uint32_t)c.child;
        if (qc.link != want) { std::printf("leaf link %zu/%d\n", i, k); return 1; }
        ++leaves;
        for (int t = c.child; t < c.child + c.count; ++t) {
          ++seen[t];
          const uint32_t src = bvh.order[t];
          for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 3; ++d) {
              const float x = V[3 * (size_t)I[3 * (size_t)src + v] + d];
              if (x < c.lo[d] || x > c.hi[d]) { std::printf("triangle outside leaf box\n"); return 1; }
            }
        }
      }
      for (int d = 0; d < 3; ++d) {
        const float lo = add_rounded(qn.origin[d], qc.lo[d], false);
        const float hi = add_rounded(qn.origin[d], qc.hi[d], true);
        if (!(lo <= c.lo[d]) || !(hi >= c.hi[d])) {
          std::printf("decoded box %zu/%d axis %d does not enclose: [%g, %g] vs [%g, %g]\n", i, k, d, lo, hi,
                      c.lo[d], c.hi[d]);
          return 1;
        }
        const double extent = std::fmax(1e-30, (double)hi_n[d] - lo_n[d]);
        if (std::isfinite(hi))
          max_slack = std::fmax(max_slack, ((double)c.lo[d] - lo + (double)hi - c.hi[d]) / extent);
      }
    }
  }
  for (size_t t = 0; t < nt; ++t)
    if (seen[t] != 1) { std::printf("triangle %zu in %d leaves\n", t, seen[t]); return 1; }
  // FNV-1a over the wide nodes, the triangle order and the depth: the tree's identity
  uint64_t hash = 1469598103934665603ull;
  auto mix = [&hash](const void *p, size_t bytes) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < bytes; ++i) hash = (hash ^ c[i]) * 1099511628211ull;
  };
  mix(bvh.nodes.data(), sizeof(BvhNode) * bvh.nodes.size());
  mix(bvh.order.data(), sizeof(uint32_t) * bvh.order.size());
  mix(&bvh.depth, sizeof bvh.depth);
  std::printf("nodes %zu depth %d leaves %zu max_slack %.3g sah_nodes %.6g sah_tris %.6g hash %016llx\n",
              bvh.nodes.size(), bvh.depth, leaves, max_slack, bvh.sah_node_visits, bvh.sah_triangle_tests,
              (unsigned long long)hash);
  return 0;
}
