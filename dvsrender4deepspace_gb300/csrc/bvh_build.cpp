// Host builder of the 8-wide BVH.
//
// Replaces the reference's single-threaded recursive binned-SAH builder
// (src/bvh/build.cpp:27-174, src/bvh/bining.cpp:9-182).  Design:
//   1. triangle centroids -> 63-bit Morton codes on one uniform grid (so a
//      flat terrain splits on x/y first, not on its thin z range);
//   2. parallel LSD radix sort of (code, triangle);
//   3. top-down radix splits at the highest differing code bit, giving a
//      binary tree over contiguous leaf ranges (<= leaf_size triangles);
//   4. collapse to 8-wide nodes -- by default choosing the wide nodes by
//      surface-area cost over slot budgets (plan_slots; 1.3 % faster traces
//      and 27 % fewer nodes than opening the largest-area inner child
//      greedily, collapse 0); nodes are numbered breadth-first so the top
//      levels are first.
// All passes are O(n) or O(n log n) and OpenMP-parallel; this is builder 1.
// The default, builder 0, replaces the Morton steps 2-3 by binned SAH splits
// with the reference's criterion (SahBuilder) and shares step 4, so the two
// trees differ only in where they split (the SAH tree traces 5 % faster on
// the 4096^2 terrain at 1280x720); both report the surface-area model of the
// wide tree.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "dvs_internal.h"

namespace dvsgb {
namespace {

struct Box {
  float lo[3], hi[3];
};
inline Box empty_box() {
  const float inf = std::numeric_limits<float>::infinity();
  return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}
inline void grow(Box &b, const Box &o) {
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = std::min(b.lo[d], o.lo[d]);
    b.hi[d] = std::max(b.hi[d], o.hi[d]);
  }
}
inline float half_area(const Box &b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// Spreads the low 21 bits of v so that two zero bits separate each.
inline uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x001f00000000ffffull;
  v = (v | (v << 16)) & 0x001f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

int thread_count() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// LSD radix sort of 64-bit keys with 32-bit payloads, 11-bit digits.
void radix_sort(std::vector<uint64_t> &keys, std::vector<uint32_t> &vals) {
  const size_t n = keys.size();
  std::vector<uint64_t> k2(n);
  std::vector<uint32_t> v2(n);
  const int bits = 11, buckets = 1 << bits;
  const int nt = std::max(1, std::min(thread_count(), int(n / 65536) + 1));
  std::vector<size_t> hist((size_t)nt * buckets);
  uint64_t all_or = 0, all_and = ~0ull;
  for (size_t i = 0; i < n; ++i) { all_or |= keys[i]; all_and &= keys[i]; }
  for (int shift = 0; shift < 64; shift += bits) {
    const uint64_t digit_mask = (uint64_t(buckets) - 1) << shift;
    if (((all_or ^ all_and) & digit_mask) == 0) continue;  // digit identical everywhere
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num();
#else
      const int t = 0;
#endif
      const size_t b = n * t / nt, e = n * (t + 1) / nt;
      size_t *h = &hist[(size_t)t * buckets];
      for (size_t i = b; i < e; ++i) h[(keys[i] >> shift) & (buckets - 1)]++;
#pragma omp barrier
#pragma omp single
      {
        size_t sum = 0;
        for (int d = 0; d < buckets; ++d)
          for (int tt = 0; tt < nt; ++tt) {
            size_t c = hist[(size_t)tt * buckets + d];
            hist[(size_t)tt * buckets + d] = sum;
            sum += c;
          }
      }
      for (size_t i = b; i < e; ++i) {
        size_t pos = h[(keys[i] >> shift) & (buckets - 1)]++;
        k2[pos] = keys[i];
        v2[pos] = vals[i];
      }
    }
    keys.swap(k2);
    vals.swap(v2);
  }
}

struct BinNode {
  Box box;
  int32_t left, right;  // -1 for leaves
  int32_t start, count;
  float area;
};

struct TreeBuilder {
  const std::vector<uint64_t> &codes;
  const std::vector<Box> &tri_boxes;  // in sorted order
  std::vector<BinNode> &nodes;
  std::atomic<int32_t> next{0};
  int leaf_size;

  int32_t build(int32_t b, int32_t e) {
    const int32_t id = next.fetch_add(1);
    BinNode &n = nodes[id];
    if (e - b <= leaf_size) {
      Box box = empty_box();
      for (int32_t i = b; i < e; ++i) grow(box, tri_boxes[i]);
      n.box = box;
      n.left = n.right = -1;
      n.start = b;
      n.count = e - b;
      n.area = half_area(box);
      return id;
    }
    int32_t m;
    const uint64_t a = codes[b], z = codes[e - 1];
    if (a == z) {
      m = b + (e - b) / 2;
    } else {
      const int h = 63 - __builtin_clzll(a ^ z);
      // first index in [b, e) whose bit h is set (codes are sorted)
      int32_t lo = b, hi = e - 1;
      while (lo < hi) {
        int32_t mid = lo + (hi - lo) / 2;
        if ((codes[mid] >> h) & 1) hi = mid; else lo = mid + 1;
      }
      m = lo;
    }
    int32_t l, r;
    if (e - b > 32768) {
#pragma omp task shared(l)
      l = build(b, m);
#pragma omp task shared(r)
      r = build(m, e);
#pragma omp taskwait
    } else {
      l = build(b, m);
      r = build(m, e);
    }
    BinNode &nn = nodes[id];
    nn.box = nodes[l].box;
    grow(nn.box, nodes[r].box);
    nn.left = l;
    nn.right = r;
    nn.start = 0;
    nn.count = 0;
    nn.area = half_area(nn.box);
    return id;
  }
};

// ---- binned SAH splits (builder 0, the default) --------------------------------------
// The reference's split criterion (src/bvh/bining.cpp:9-103): over the
// centroid bounds of a range, min(32, 4 + 0.05 n) bins per axis; each
// triangle's box grows the bin of its centroid; at every bin boundary of the
// three axes the cost area(left) * n_left + area(right) * n_right, the least
// taken (first axis, then first boundary, on ties).  Unlike the reference a
// range is always split down to leaf_size triangles: the leaves here have a
// fixed maximum size and the 8-wide collapse sets the node layout.  A range
// whose centroids share one bin on every axis is halved by index.  Large
// ranges scan their references in parallel chunks; subtrees of more than
// 32768 triangles are OpenMP tasks.
struct SahRef {
  Box box;
  float c[3];
  uint32_t id;
};
constexpr int kSahBins = 32;

struct SahBuilder {
  std::vector<SahRef> &refs;
  std::vector<BinNode> &nodes;
  std::atomic<int32_t> next{0};
  int leaf_size;

  static int chunks_for(int32_t n) { return n > (1 << 20) ? std::max(1, std::min(4 * thread_count(), n >> 18)) : 1; }
  static int32_t chunk_begin(int32_t b, int32_t n, int k, int chunks) {
    return b + (int32_t)((int64_t)n * k / chunks);
  }
  static int bin_of(float c, float lo, float scale, int nb) {
    const int j = (int)((c - lo) * scale);
    return std::min(std::max(j, 0), nb - 1);
  }

  // box of the range and bounds of its centroids
  void bounds(int32_t b, int32_t e, Box &range, Box &cent) {
    const int32_t n = e - b;
    const int chunks = chunks_for(n);
    std::vector<Box> pr(chunks), pc(chunks);
    for (int k = 0; k < chunks; ++k) {
#pragma omp task shared(pr, pc) firstprivate(k) if (chunks > 1)
      {
        Box r = empty_box(), c = empty_box();
        for (int32_t i = chunk_begin(b, n, k, chunks), ie = chunk_begin(b, n, k + 1, chunks); i < ie; ++i) {
          grow(r, refs[i].box);
          for (int d = 0; d < 3; ++d) {
            c.lo[d] = std::min(c.lo[d], refs[i].c[d]);
            c.hi[d] = std::max(c.hi[d], refs[i].c[d]);
          }
        }
        pr[k] = r;
        pc[k] = c;
      }
    }
#pragma omp taskwait
    range = cent = empty_box();
    for (int k = 0; k < chunks; ++k) {
      grow(range, pr[k]);
      grow(cent, pc[k]);
    }
  }

  // Per axis and bin: the union of the triangles' boxes, the bounds of their
  // centroids, and their count.  A split's two sides are unions of bins, so
  // the children's boxes and centroid bounds come from the bins: the same
  // minima and maxima a scan of the children's triangles would give, without
  // the scan.
  struct Bins {
    Box box[3][kSahBins];
    Box cent[3][kSahBins];
    int32_t count[3][kSahBins];
    void clear() {
      for (int d = 0; d < 3; ++d)
        for (int j = 0; j < kSahBins; ++j) {
          box[d][j] = cent[d][j] = empty_box();
          count[d][j] = 0;
        }
    }
  };

  // Range [b, e) with its box and its centroids' bounds.
  int32_t build(int32_t b, int32_t e, Box range, Box cent) {
    const int32_t id = next.fetch_add(1);
    const int32_t n = e - b;
    if (n <= leaf_size) {
      BinNode &leaf = nodes[id];
      leaf.box = range;
      leaf.left = leaf.right = -1;
      leaf.start = b;
      leaf.count = n;
      leaf.area = half_area(range);
      return id;
    }
    const int nb = std::min(kSahBins, (int)(4.0f + 0.05f * (float)n));
    float scale[3];
    for (int d = 0; d < 3; ++d) {
      const float extent = cent.hi[d] - cent.lo[d];
      scale[d] = extent > 0 ? (float)nb / extent : 0.0f;
    }
    // bin the range (chunks in parallel for large ranges)
    const int chunks = chunks_for(n);
    std::vector<Bins> part(chunks);
    for (int k = 0; k < chunks; ++k) {
#pragma omp task shared(part, scale, cent) firstprivate(k) if (chunks > 1)
      {
        Bins &p = part[k];
        p.clear();
        for (int32_t i = chunk_begin(b, n, k, chunks), ie = chunk_begin(b, n, k + 1, chunks); i < ie; ++i) {
          const SahRef &ref = refs[i];
          const Box point{{ref.c[0], ref.c[1], ref.c[2]}, {ref.c[0], ref.c[1], ref.c[2]}};
          for (int d = 0; d < 3; ++d) {
            const int j = bin_of(ref.c[d], cent.lo[d], scale[d], nb);
            grow(p.box[d][j], ref.box);
            grow(p.cent[d][j], point);
            ++p.count[d][j];
          }
        }
      }
    }
#pragma omp taskwait
    Bins &bins = part[0];
    for (int k = 1; k < chunks; ++k)
      for (int d = 0; d < 3; ++d)
        for (int j = 0; j < nb; ++j) {
          grow(bins.box[d][j], part[k].box[d][j]);
          grow(bins.cent[d][j], part[k].cent[d][j]);
          bins.count[d][j] += part[k].count[d][j];
        }
    // sweep every boundary of every axis
    float best = std::numeric_limits<float>::infinity();
    int best_d = -1, best_j = 0;
    for (int d = 0; d < 3; ++d) {
      Box right[kSahBins];
      int32_t right_n[kSahBins];
      Box acc = empty_box();
      int32_t acc_n = 0;
      for (int j = nb - 1; j >= 0; --j) {
        grow(acc, bins.box[d][j]);
        acc_n += bins.count[d][j];
        right[j] = acc;
        right_n[j] = acc_n;
      }
      Box left = empty_box();
      int32_t left_n = 0;
      for (int j = 1; j < nb; ++j) {
        grow(left, bins.box[d][j - 1]);
        left_n += bins.count[d][j - 1];
        if (left_n == 0 || right_n[j] == 0) continue;
        const float cost = half_area(left) * (float)left_n + half_area(right[j]) * (float)right_n[j];
        if (cost < best) {
          best = cost;
          best_d = d;
          best_j = j;
        }
      }
    }
    int32_t m;
    Box lrange, lcent, rrange, rcent;
    if (best_d >= 0) {
      // the same bin_of as the binning pass, so the split has the swept counts
      const int d = best_d;
      const float lo = cent.lo[d], sc = scale[d];
      m = (int32_t)(std::partition(refs.begin() + b, refs.begin() + e,
                                   [&](const SahRef &r) { return bin_of(r.c[d], lo, sc, nb) < best_j; }) -
                    refs.begin());
      lrange = lcent = rrange = rcent = empty_box();
      for (int j = 0; j < nb; ++j) {
        grow(j < best_j ? lrange : rrange, bins.box[d][j]);
        grow(j < best_j ? lcent : rcent, bins.cent[d][j]);
      }
    } else {
      m = b + n / 2;  // every centroid in one bin on every axis
      bounds(b, m, lrange, lcent);
      bounds(m, e, rrange, rcent);
    }
    int32_t l, r;
    if (n > 32768) {
#pragma omp task shared(l, lrange, lcent)
      l = build(b, m, lrange, lcent);
#pragma omp task shared(r, rrange, rcent)
      r = build(m, e, rrange, rcent);
#pragma omp taskwait
    } else {
      l = build(b, m, lrange, lcent);
      r = build(m, e, rrange, rcent);
    }
    BinNode &nn = nodes[id];
    nn.box = range;
    nn.left = l;
    nn.right = r;
    nn.start = 0;
    nn.count = 0;
    nn.area = half_area(range);
    return id;
  }
};

// ---- 8-wide collapse by slot budgets (collapse 1) -----------------------------------
// D(b, j), j = 1..8: the least surface-area cost of covering binary subtree b
// with at most j children of one wide node.  A binary leaf as a child costs
// kTriCost x area x triangles; an inner node as one child is a wide node of its
// own, kNodeCost x area + S(b, 8); with j >= 2 slots the subtree may instead be
// split between its two children, S(b, j) = min over k of D(left, k) +
// D(right, j - k).  The wide node made from inner node b takes the children of
// S(b, 8).  A node's tables need its children's: they are filled in post
// order, the subtrees of the top levels as parallel tasks.  (Areas are the binary boxes' half areas;
// the ratio to the root's area is the probability a ray enters the box.)
constexpr float kNodeCost = 1.0f, kTriCost = 1.0f;
struct SlotPlan {
  std::vector<float> d;       // D(b, j) at 8 * b + j - 1
  std::vector<uint8_t> pick;  // for j >= 2: 0 = b itself as one child, k = k slots to the left
  std::vector<uint8_t> wide;  // k of S(b, 8), the split the wide node made from b uses
  void emit(const std::vector<BinNode> &bin, int32_t b, int j, int32_t *kids, int &nk) const {
    const int k = (bin[b].count > 0 || j == 1) ? 0 : pick[8 * (size_t)b + j - 1];
    if (k == 0) {
      kids[nk++] = b;
      return;
    }
    emit(bin, bin[b].left, k, kids, nk);
    emit(bin, bin[b].right, j - k, kids, nk);
  }
  void children(const std::vector<BinNode> &bin, int32_t b, int32_t *kids, int &nk) const {
    const int k = wide[b];
    emit(bin, bin[b].left, k, kids, nk);
    emit(bin, bin[b].right, kBvhWidth - k, kids, nk);
  }
};
// D(i, .) of one node from its children's (already filled).
void plan_node(const std::vector<BinNode> &bin, SlotPlan &p, size_t i) {
  const BinNode &b = bin[i];
  float *d = &p.d[8 * i];
  if (b.count > 0) {
    const float leaf = kTriCost * b.area * (float)b.count;
    for (int j = 0; j < 8; ++j) d[j] = leaf;
    return;
  }
  const float *dl = &p.d[8 * (size_t)b.left], *dr = &p.d[8 * (size_t)b.right];
  float s[9];  // S(b, j), j = 2..8
  uint8_t sk[9];
  for (int j = 2; j <= 8; ++j) {
    s[j] = std::numeric_limits<float>::infinity();
    sk[j] = 1;
    for (int k = 1; k < j; ++k) {
      const float c = dl[k - 1] + dr[j - k - 1];
      if (c < s[j]) { s[j] = c; sk[j] = (uint8_t)k; }
    }
  }
  p.wide[i] = sk[8];
  d[0] = kNodeCost * b.area + s[8];
  for (int j = 2; j <= 8; ++j) {
    if (s[j] < d[0]) {
      d[j - 1] = s[j];
      p.pick[8 * i + j - 1] = sk[j];
    } else {
      d[j - 1] = d[0];
      p.pick[8 * i + j - 1] = 0;
    }
  }
}
// Children before their parent; the top levels' subtrees as parallel tasks.
void plan_subtree(const std::vector<BinNode> &bin, SlotPlan &p, int32_t i, int depth) {
  const BinNode &b = bin[i];
  if (b.count == 0) {
    if (depth < 12) {
#pragma omp task shared(bin, p)
      plan_subtree(bin, p, b.left, depth + 1);
#pragma omp task shared(bin, p)
      plan_subtree(bin, p, b.right, depth + 1);
#pragma omp taskwait
    } else {
      plan_subtree(bin, p, b.left, depth + 1);
      plan_subtree(bin, p, b.right, depth + 1);
    }
  }
  plan_node(bin, p, (size_t)i);
}
SlotPlan plan_slots(const std::vector<BinNode> &bin, int32_t root) {
  SlotPlan p;
  const size_t n = bin.size();
  p.d.assign(8 * n, 0.0f);
  p.pick.assign(8 * n, 0);
  p.wide.assign(n, 1);
#pragma omp parallel
#pragma omp single
  plan_subtree(bin, p, root, 0);
  return p;
}

}  // namespace

bool build_bvh(const float *V, size_t nv, const uint32_t *I, size_t nt, int leaf_size, int builder, BvhBuild &out,
               std::string &error, int collapse) {
  const auto t_start = std::chrono::steady_clock::now();
  if (nt == 0 || nv == 0) { error = "empty mesh"; return false; }
  if (nt > (size_t(1) << 28)) { error = "mesh exceeds 2^28 triangles"; return false; }
  if (leaf_size < 1 || leaf_size > 8) { error = "leaf_size must be 1..8"; return false; }
  if (builder != 0 && builder != 1) { error = "BVH builder must be 0 (binned SAH) or 1 (Morton radix)"; return false; }
  for (size_t i = 0; i < 3 * nt; ++i)
    if (I[i] >= nv) { error = "mesh triangle index outside vertex array"; return false; }

  // 1. bounds and Morton codes
  std::vector<Box> boxes(nt);
  Box scene = empty_box();
  const long long ntl = (long long)nt;
#pragma omp parallel
  {
    Box local = empty_box();
#pragma omp for schedule(static)
    for (long long i = 0; i < ntl; ++i) {
      Box b = empty_box();
      for (int k = 0; k < 3; ++k) {
        const float *p = V + 3 * (size_t)I[3 * i + k];
        for (int d = 0; d < 3; ++d) { b.lo[d] = std::min(b.lo[d], p[d]); b.hi[d] = std::max(b.hi[d], p[d]); }
      }
      boxes[i] = b;
      Box c;
      for (int d = 0; d < 3; ++d) c.lo[d] = c.hi[d] = 0.5f * (b.lo[d] + b.hi[d]);
      grow(local, c);
    }
#pragma omp critical
    grow(scene, local);
  }
  std::vector<uint32_t> order(nt);
  std::vector<BinNode> bin(2 * nt + 1);
  int32_t root = 0;
  if (builder == 0) {
    // 2-3. binned SAH splits over the triangles' boxes and centroids
    std::vector<SahRef> refs(nt);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < ntl; ++i) {
      refs[i].box = boxes[i];
      for (int d = 0; d < 3; ++d) refs[i].c[d] = 0.5f * (boxes[i].lo[d] + boxes[i].hi[d]);
      refs[i].id = uint32_t(i);
    }
    std::vector<Box>().swap(boxes);
    SahBuilder sb{refs, bin, {}, leaf_size};
#pragma omp parallel
#pragma omp single
    {
      Box range, cent;
      sb.bounds(0, (int32_t)nt, range, cent);
      root = sb.build(0, (int32_t)nt, range, cent);
    }
    bin.resize(sb.next.load());
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < ntl; ++i) order[i] = refs[i].id;
  } else {
    float extent = std::max({scene.hi[0] - scene.lo[0], scene.hi[1] - scene.lo[1], scene.hi[2] - scene.lo[2]});
    if (!(extent > 0) || !std::isfinite(extent)) extent = 1.0f;
    const double scale = double((1u << 21) - 1) / double(extent);
    std::vector<uint64_t> codes(nt);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < ntl; ++i) {
      uint64_t q[3];
      for (int d = 0; d < 3; ++d) {
        double c = 0.5 * (double(boxes[i].lo[d]) + double(boxes[i].hi[d]));
        double v = (c - scene.lo[d]) * scale;
        v = std::min(std::max(v, 0.0), double((1u << 21) - 1));
        q[d] = uint64_t(v);
      }
      codes[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
      order[i] = uint32_t(i);
    }

    // 2. sort
    radix_sort(codes, order);
    std::vector<Box> sorted_boxes(nt);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < ntl; ++i) sorted_boxes[i] = boxes[order[i]];
    std::vector<Box>().swap(boxes);

    // 3. binary radix tree
    TreeBuilder tb{codes, sorted_boxes, bin, {}, leaf_size};
#pragma omp parallel
#pragma omp single
    root = tb.build(0, (int32_t)nt);
    bin.resize(tb.next.load());
  }

  // 4. collapse to kBvhWidth-wide, breadth first: level by level, each level's
  // wide nodes in parallel; a prefix sum of their inner children numbers the
  // next level in the order a serial breadth-first queue would
  const SlotPlan plan = collapse == 1 ? plan_slots(bin, root) : SlotPlan{};
  std::vector<BvhNode> nodes;
  nodes.reserve(bin.size() / (kBvhWidth - 1) + 2);
  std::vector<int32_t> level{root};  // binary node per wide node of the level
  int depth = 0;
  while (!level.empty()) {
    ++depth;
    const long long m = (long long)level.size();
    const size_t base = nodes.size();
    nodes.resize(base + (size_t)m);
    std::vector<int32_t> kids_of((size_t)m * kBvhWidth);
    std::vector<int> nk_of((size_t)m);
    std::vector<long long> inner_at((size_t)m + 1, 0);  // inner children before wide node q of the level
#pragma omp parallel for schedule(static) if (m > 4096)
    for (long long q = 0; q < m; ++q) {
      const int32_t b = level[q];
      int32_t *kids = &kids_of[(size_t)q * kBvhWidth];
      int nk = 0;
      if (bin[b].count > 0) {
        kids[nk++] = b;  // a leaf root: one leaf child
      } else if (collapse == 1) {
        plan.children(bin, b, kids, nk);
      } else {
        kids[nk++] = bin[b].left;
        kids[nk++] = bin[b].right;
        while (nk < kBvhWidth) {
          int best = -1;
          float best_area = -1;
          for (int k = 0; k < nk; ++k)
            if (bin[kids[k]].count == 0 && bin[kids[k]].area > best_area) { best = k; best_area = bin[kids[k]].area; }
          if (best < 0) break;
          const int32_t open = kids[best];
          kids[best] = bin[open].left;
          kids[nk++] = bin[open].right;
        }
      }
      nk_of[q] = nk;
      int inner = 0;
      for (int k = 0; k < nk; ++k) inner += bin[kids[k]].count > 0 ? 0 : 1;
      inner_at[q + 1] = inner;
    }
    for (long long q = 0; q < m; ++q) inner_at[q + 1] += inner_at[q];
    const size_t next_base = base + (size_t)m;
    std::vector<int32_t> next((size_t)inner_at[m]);
#pragma omp parallel for schedule(static) if (m > 4096)
    for (long long q = 0; q < m; ++q) {
      const int32_t *kids = &kids_of[(size_t)q * kBvhWidth];
      const int nk = nk_of[q];
      long long slot = inner_at[q];
      BvhNode node;
      std::memset(&node, 0, sizeof(node));
      for (int k = 0; k < kBvhWidth; ++k) {
        BvhChild &out_child = node.c[k];
        if (k >= nk) {
          out_child.child = -1;
          out_child.count = -1;
          continue;
        }
        const BinNode &c = bin[kids[k]];
        for (int d = 0; d < 3; ++d) { out_child.lo[d] = c.box.lo[d]; out_child.hi[d] = c.box.hi[d]; }
        if (c.count > 0) {
          out_child.child = c.start;
          out_child.count = c.count;
        } else {
          out_child.child = (int32_t)(next_base + (size_t)slot);
          out_child.count = 0;
          next[(size_t)slot++] = kids[k];
        }
      }
      nodes[base + (size_t)q] = node;
    }
    level.swap(next);
  }
  if ((kBvhWidth - 1) * depth + 1 > kStackSlots) {
    error = "BVH too deep for the traversal stack (depth " + std::to_string(depth) + ")";
    return false;
  }
  // Surface-area model of the wide tree: a ray through the root box enters a
  // box with probability area(box) / area(root), so the expected wide nodes
  // visited is the sum of the nodes' areas and the expected triangle tests the
  // sum of leaf area x triangles, both over the root's area (double sums).
  {
    auto child_box = [](const BvhChild &c) {
      Box b;
      for (int d = 0; d < 3; ++d) { b.lo[d] = c.lo[d]; b.hi[d] = c.hi[d]; }
      return b;
    };
    auto node_area = [&](const BvhNode &nd) {
      Box b = empty_box();
      for (int k = 0; k < kBvhWidth; ++k)
        if (nd.c[k].count >= 0) grow(b, child_box(nd.c[k]));
      return (double)half_area(b);
    };
    const double root_area = node_area(nodes[0]);
    double visits = 0, tests = 0;
    for (const BvhNode &nd : nodes) {
      visits += node_area(nd);
      for (int k = 0; k < kBvhWidth; ++k)
        if (nd.c[k].count > 0) tests += (double)half_area(child_box(nd.c[k])) * nd.c[k].count;
    }
    out.sah_node_visits = root_area > 0 ? visits / root_area : 0;
    out.sah_triangle_tests = root_area > 0 ? tests / root_area : 0;
  }
  out.nodes.swap(nodes);
  out.order.swap(order);
  out.depth = depth;
  out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return true;
}

// ---- precision-format nodes -------------------------------------------------------
namespace {
// FP16 bits of the largest half <= x (up = false) or the smallest half >= x
// (up = true), for finite x >= 0.  Beyond the largest finite half (65504) the
// lower bound saturates and the upper bound becomes +inf, both conservative.
uint16_t half_directed(double x, bool up) {
  if (!(x > 0.0)) return 0;
  if (x > 65504.0) return up ? 0x7c00 : 0x7bff;
  int e = 0;
  std::frexp(x, &e);          // x in [2^(e-1), 2^e)
  const int E = e + 14;       // biased half exponent of that binade
  uint32_t bits;
  if (E <= 0) {               // subnormal: units of 2^-24
    const double u = std::ldexp(x, 24);
    bits = (uint32_t)(up ? std::ceil(u) : std::floor(u));
  } else {                    // normal: (1024 + mantissa) * 2^(E - 25)
    const double u = std::ldexp(x, 25 - E);
    bits = ((uint32_t)E << 10) + ((uint32_t)(up ? std::ceil(u) : std::floor(u)) - 1024u);  // 2048 carries
  }
  if (bits >= 0x7c00u) bits = up ? 0x7c00u : 0x7bffu;
  return (uint16_t)bits;
}
double half_value(uint16_t h) {
  const int E = (h >> 10) & 31, m = h & 1023;
  if (E == 31) return m ? std::numeric_limits<double>::quiet_NaN() : std::numeric_limits<double>::infinity();
  return E == 0 ? std::ldexp((double)m, -24) : std::ldexp((double)(1024 + m), E - 25);
}
// origin + offset rounded to float toward -inf / +inf, as __fadd_rd/__fadd_ru.
// The exact sum is s + err (Knuth's TwoSum in double).
float add_directed(float origin, uint16_t off, bool up) {
  const double a = origin, b = half_value(off);
  const double s = a + b;
  if (std::isinf(s)) return (float)s;
  const double bb = s - a, err = (a - (s - bb)) + (b - bb);
  float f = (float)s;
  const double fd = f;
  if (!up && (fd > s || (fd == s && err < 0))) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
  if (up && (fd < s || (fd == s && err > 0))) f = std::nextafter(f, std::numeric_limits<float>::infinity());
  return f;
}
}  // namespace

bool quantize_bvh(const std::vector<BvhNode> &nodes, std::vector<BvhQNode> &out, std::string &error) {
  out.assign(nodes.size(), BvhQNode{});
  std::atomic<bool> bad_link{false}, bad_box{false};
  const long long n = (long long)nodes.size();
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) {
    const BvhNode &src = nodes[i];
    BvhQNode &q = out[i];
    float origin[3] = {0.0f, 0.0f, 0.0f};
    bool any = false;
    for (int k = 0; k < kBvhWidth; ++k) {
      if (src.c[k].count < 0) continue;
      for (int d = 0; d < 3; ++d) origin[d] = any ? std::min(origin[d], src.c[k].lo[d]) : src.c[k].lo[d];
      any = true;
    }
    for (int d = 0; d < 3; ++d) q.origin[d] = origin[d];
    q.pad = 0;
    for (int k = 0; k < kBvhWidth; ++k) {
      const BvhChild &c = src.c[k];
      BvhQChild &qc = q.c[k];
      if (c.count < 0) {
        for (int d = 0; d < 3; ++d) qc.lo[d] = qc.hi[d] = 0x7c00;
        qc.link = kQLinkEmpty;
        continue;
      }
      for (int d = 0; d < 3; ++d) {
        qc.lo[d] = half_directed((double)c.lo[d] - (double)origin[d], false);
        qc.hi[d] = half_directed((double)c.hi[d] - (double)origin[d], true);
        if (!(add_directed(origin[d], qc.lo[d], false) <= c.lo[d]) ||
            !(add_directed(origin[d], qc.hi[d], true) >= c.hi[d]))
          bad_box = true;
      }
      if (c.count == 0) {
        qc.link = (uint32_t)c.child;
      } else if (c.count > 16 || (uint64_t)c.child + (uint64_t)c.count > (uint64_t)kQLinkFirstMask + 1) {
        bad_link = true;
        qc.link = kQLinkEmpty;
      } else {
        qc.link = kQLinkLeaf | ((uint32_t)(c.count - 1) << kQLinkCountShift) | (uint32_t)c.child;
      }
    }
  }
  if (bad_link) {
    error = "mesh too large for the precision BVH format (more than 2^27 triangles)";
    return false;
  }
  if (bad_box) {
    error = "quantised BVH bounds do not enclose the FP32 bounds";
    return false;
  }
  return true;
}

}  // namespace dvsgb
