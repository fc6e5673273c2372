// bvh_sah.cpp -- binned-SAH hierarchy over scene triangles, built on the host.
//
// The reference leaves hierarchy quality to the OptiX GAS builder
// (optixPathTracer.cpp:382-450).  A Morton-code LBVH splits at fixed spatial
// planes; on scenes of tens of thousands of triangles (rooms full of
// tessellated obstacles, multi-room buildings) its closest-hit queries visit
// 30-60% more nodes than a surface-area-heuristic tree.  This builder makes
// the SAH tree once per scene:
//   * top-down binned SAH (32 bins per axis, cost = area x count of both
//     sides, Wald 2007 "On fast construction of SAH-based BVHs"), one
//     primitive per leaf;
//   * below depth 32 the split is the object median of the widest centroid
//     axis, so the depth stays under 32 + 28 and the 64-entry traversal stack
//     of the kernels never overflows;
//   * an internal node is numbered by its split position (the boundary
//     between sorted leaves mid-1 and mid belongs to exactly one node), so
//     subtrees are built on separate threads without coordination; a
//     depth-first pass then renumbers the nodes with the root at 0 and each
//     subtree contiguous;
//   * child boxes are widened outward exactly as the GPU refit widens them,
//     so node culling stays conservative and the closest hit (chosen by t,
//     instance, original primitive index) does not depend on the tree.
#include "bvh_sah.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <exception>
#include <thread>

namespace {

struct Bx {
  float lo[3], hi[3];
};

inline Bx bx_empty() {
  Bx b;
  for (int k = 0; k < 3; k++) { b.lo[k] = 3.0e38f; b.hi[k] = -3.0e38f; }
  return b;
}

inline void bx_grow(Bx &a, const Bx &b) {
  for (int k = 0; k < 3; k++) {
    a.lo[k] = std::min(a.lo[k], b.lo[k]);
    a.hi[k] = std::max(a.hi[k], b.hi[k]);
  }
}

inline double half_area(const Bx &b) {
  const double dx = (double)b.hi[0] - b.lo[0], dy = (double)b.hi[1] - b.lo[1],
               dz = (double)b.hi[2] - b.lo[2];
  if (dx < 0.0) return 0.0;
  return dx * dy + dy * dz + dz * dx;
}

inline float widen_lo(float v) {
  return std::nextafter(v - (1e-6f + 1e-6f * std::fabs(v)), -3.0e38f);
}
inline float widen_hi(float v) {
  return std::nextafter(v + (1e-6f + 1e-6f * std::fabs(v)), 3.0e38f);
}

constexpr int kBins = 32;
constexpr int kSahDepth = 32;
constexpr int kParallelMin = 8192;

struct Builder {
  const Bx *box;
  const float *cen;  // 3 per primitive
  int *idx;          // primitive order, partitioned in place
  int *child;        // [2 * split id]: child references of each internal node
  Bx *cbox;          // [2 * split id]: child boxes

  // bin of centroid coordinate c on an axis starting at lo with kBins / ext
  static inline int bin_of(float c, float lo, float scale) {
    int b = (int)((c - lo) * scale);
    return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
  }

  // builds idx[lo, hi); returns the reference of the subtree root and its box
  int build(int lo, int hi, int depth, int spawn, Bx &out, int &out_depth) {
    if (hi - lo == 1) {
      out = box[idx[lo]];
      out_depth = depth;
      return ~lo;
    }
    Bx cb = bx_empty();
    for (int i = lo; i < hi; i++) {
      const float *c = cen + 3 * idx[i];
      for (int k = 0; k < 3; k++) {
        cb.lo[k] = std::min(cb.lo[k], c[k]);
        cb.hi[k] = std::max(cb.hi[k], c[k]);
      }
    }
    int mid = -1;
    if (depth < kSahDepth) {
      double best = 1e300;
      int bax = -1, bsplit = 0;
      for (int ax = 0; ax < 3; ax++) {
        const float ext = cb.hi[ax] - cb.lo[ax];
        if (!(ext > 0.0f)) continue;
        const float scale = (float)kBins / ext;
        Bx bb[kBins];
        int cnt[kBins];
        for (int b = 0; b < kBins; b++) { bb[b] = bx_empty(); cnt[b] = 0; }
        for (int i = lo; i < hi; i++) {
          const int p = idx[i];
          const int b = bin_of(cen[3 * p + ax], cb.lo[ax], scale);
          cnt[b]++;
          bx_grow(bb[b], box[p]);
        }
        double left_cost[kBins];
        int left_n[kBins];
        Bx acc = bx_empty();
        int c = 0;
        for (int b = 0; b < kBins - 1; b++) {
          bx_grow(acc, bb[b]);
          c += cnt[b];
          left_cost[b] = half_area(acc) * c;
          left_n[b] = c;
        }
        acc = bx_empty();
        c = 0;
        for (int b = kBins - 1; b > 0; b--) {
          bx_grow(acc, bb[b]);
          c += cnt[b];
          if (left_n[b - 1] == 0 || c == 0) continue;
          const double cost = left_cost[b - 1] + half_area(acc) * c;
          if (cost < best) { best = cost; bax = ax; bsplit = b; }
        }
      }
      if (bax >= 0) {
        const float lo_ax = cb.lo[bax], scale = (float)kBins / (cb.hi[bax] - cb.lo[bax]);
        int *m = std::partition(idx + lo, idx + hi, [&](int p) {
          return bin_of(cen[3 * p + bax], lo_ax, scale) < bsplit;
        });
        mid = (int)(m - idx);
        if (mid <= lo || mid >= hi) mid = -1;
      }
    }
    if (mid < 0) {
      // object median of the widest centroid axis (all centroids equal: any
      // split of the index range)
      int ax = 0;
      for (int k = 1; k < 3; k++)
        if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
      mid = lo + (hi - lo) / 2;
      if (cb.hi[ax] - cb.lo[ax] > 0.0f)
        std::nth_element(idx + lo, idx + mid, idx + hi,
                         [&](int a, int b) { return cen[3 * a + ax] < cen[3 * b + ax]; });
    }
    const int id = mid - 1;
    Bx b0, b1;
    int d0 = 0, d1 = 0, r0 = 0, r1 = 0;
    std::thread th;
    bool spawned = false;
    if (spawn > 0 && hi - lo >= kParallelMin) {
      try {
        th = std::thread([&] { r0 = build(lo, mid, depth + 1, spawn - 1, b0, d0); });
        spawned = true;
      } catch (...) {
        spawned = false;  // no thread available: build this side here
      }
    }
    if (!spawned) r0 = build(lo, mid, depth + 1, std::max(spawn - 1, 0), b0, d0);
    r1 = build(mid, hi, depth + 1, std::max(spawn - 1, 0), b1, d1);
    if (spawned) th.join();
    child[2 * id] = r0;
    child[2 * id + 1] = r1;
    cbox[2 * id] = b0;
    cbox[2 * id + 1] = b1;
    out = b0;
    bx_grow(out, b1);
    out_depth = std::max(d0, d1);
    return id;
  }
};

}  // namespace

static bool sah_build_impl(const float *tris, int n, std::vector<BvhNode> &nodes,
                           std::vector<int> &perm, char *msg, size_t msglen) {
  nodes.clear();
  perm.assign((size_t)std::max(n, 0), 0);
  if (n <= 0) return true;
  std::vector<Bx> box((size_t)n);
  std::vector<float> cen(3 * (size_t)n);
  for (int i = 0; i < n; i++) {
    const float *v = tris + 9 * (size_t)i;
    Bx b;
    for (int k = 0; k < 3; k++) {
      b.lo[k] = std::min(std::min(v[k], v[3 + k]), v[6 + k]);
      b.hi[k] = std::max(std::max(v[k], v[3 + k]), v[6 + k]);
      cen[3 * (size_t)i + k] = 0.5f * (b.lo[k] + b.hi[k]);
    }
    box[(size_t)i] = b;
    perm[(size_t)i] = i;
  }
  if (n == 1) return true;
  std::vector<int> child(2 * (size_t)(n - 1), 0);
  std::vector<Bx> cbox(2 * (size_t)(n - 1));
  Builder B{box.data(), cen.data(), perm.data(), child.data(), cbox.data()};
  unsigned hw = std::thread::hardware_concurrency();
  int spawn = 0;
  while ((1u << spawn) < std::max(hw, 1u) && spawn < 5) spawn++;
  Bx root_box;
  int depth = 0;
  const int root = B.build(0, n, 0, spawn, root_box, depth);
  if (depth >= 62) {
    snprintf(msg, msglen, "SAH hierarchy depth %d exceeds the traversal stack", depth);
    return false;
  }
  // depth-first renumbering: root 0, left subtree next
  std::vector<int> newid((size_t)(n - 1), -1);
  std::vector<int> stack;
  stack.reserve(128);
  stack.push_back(root);
  int next = 0;
  while (!stack.empty()) {
    const int s = stack.back();
    stack.pop_back();
    if (s < 0 || s >= n - 1 || newid[(size_t)s] >= 0) {
      snprintf(msg, msglen, "SAH hierarchy is not a tree (node %d)", s);
      return false;
    }
    newid[(size_t)s] = next++;
    if (child[2 * (size_t)s + 1] >= 0) stack.push_back(child[2 * (size_t)s + 1]);
    if (child[2 * (size_t)s] >= 0) stack.push_back(child[2 * (size_t)s]);
  }
  if (next != n - 1) {
    snprintf(msg, msglen, "SAH hierarchy reaches %d of %d internal nodes", next, n - 1);
    return false;
  }
  nodes.assign((size_t)(n - 1), BvhNode{});
  std::vector<char> leaf_seen((size_t)n, 0);
  for (int s = 0; s < n - 1; s++) {
    BvhNode &nd = nodes[(size_t)newid[(size_t)s]];
    int ref[2];
    for (int c = 0; c < 2; c++) {
      const int r = child[2 * (size_t)s + c];
      if (r < 0) {
        if (~r >= n || leaf_seen[(size_t)~r]) {
          snprintf(msg, msglen, "SAH hierarchy leaf %d is invalid or repeated", ~r);
          return false;
        }
        leaf_seen[(size_t)~r] = 1;
        ref[c] = r;
      } else {
        ref[c] = newid[(size_t)r];
      }
      const Bx &b = cbox[2 * (size_t)s + c];
      float wl[3], wh[3];
      for (int k = 0; k < 3; k++) { wl[k] = widen_lo(b.lo[k]); wh[k] = widen_hi(b.hi[k]); }
      if (c == 0) {
        nd.a = make_float4(wl[0], wl[1], wl[2], wh[0]);
        nd.b.x = wh[1];
        nd.b.y = wh[2];
      } else {
        nd.b.z = wl[0];
        nd.b.w = wl[1];
        nd.c = make_float4(wl[2], wh[0], wh[1], wh[2]);
      }
    }
    nd.d = make_int4(ref[0], ref[1], 0, 0);
  }
  return true;
}

bool sah_build_triangles(const float *tris, int n, std::vector<BvhNode> &nodes,
                         std::vector<int> &perm, char *msg, size_t msglen) {
  try {
    return sah_build_impl(tris, n, nodes, perm, msg, msglen);
  } catch (const std::exception &ex) {
    snprintf(msg, msglen, "SAH build failed: %s", ex.what());
    return false;
  }
}
