// Host-side check of the binned-SAH scene hierarchy (automs_gb300/csrc/bvh_sah.cpp),
// built by tests/test_bvh_sah.py with g++.
//
//   bvh_sah_check <triangles.bin> <n_rays> <seed>
//
// triangles.bin holds float32 [n][9].  The check builds the hierarchy and
// verifies: every internal node is reached once from the root, every leaf
// once; each child box (as stored, widened) contains its subtree's triangles;
// the depth fits the kernels' 64-entry stack; and for random rays the
// closest hit found by an ordered stack traversal of the tree (the kernels'
// order: nearer child first, far child pushed, pruned at the best t) equals a
// brute-force search over all triangles.  Prints "ok <nodes> <depth>" or the
// first failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bvh_sah.h"

namespace {

struct Box {
  float lo[3], hi[3];
};

Box child_box(const BvhNode &nd, int c) {
  Box b;
  if (c == 0) {
    b.lo[0] = nd.a.x; b.lo[1] = nd.a.y; b.lo[2] = nd.a.z;
    b.hi[0] = nd.a.w; b.hi[1] = nd.b.x; b.hi[2] = nd.b.y;
  } else {
    b.lo[0] = nd.b.z; b.lo[1] = nd.b.w; b.lo[2] = nd.c.x;
    b.hi[0] = nd.c.y; b.hi[1] = nd.c.z; b.hi[2] = nd.c.w;
  }
  return b;
}

bool contains(const Box &outer, const Box &inner) {
  for (int k = 0; k < 3; k++)
    if (inner.lo[k] < outer.lo[k] || inner.hi[k] > outer.hi[k]) return false;
  return true;
}

// Moller-Trumbore in double; t > 1e-5 or -1
double tri_t(const float *v, const double *o, const double *d) {
  double e1[3], e2[3], s[3], h[3], q[3];
  for (int k = 0; k < 3; k++) {
    e1[k] = (double)v[3 + k] - v[k];
    e2[k] = (double)v[6 + k] - v[k];
    s[k] = o[k] - v[k];
  }
  h[0] = d[1] * e2[2] - d[2] * e2[1];
  h[1] = d[2] * e2[0] - d[0] * e2[2];
  h[2] = d[0] * e2[1] - d[1] * e2[0];
  const double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
  if (std::fabs(a) < 1e-14) return -1.0;
  const double f = 1.0 / a;
  const double u = f * (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
  if (u < 0.0 || u > 1.0) return -1.0;
  q[0] = s[1] * e1[2] - s[2] * e1[1];
  q[1] = s[2] * e1[0] - s[0] * e1[2];
  q[2] = s[0] * e1[1] - s[1] * e1[0];
  const double w = f * (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]);
  if (w < 0.0 || u + w > 1.0) return -1.0;
  const double t = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
  return t > 1e-5 ? t : -1.0;
}

// slab test in double against a stored box; entry distance in tn
bool slab(const Box &b, const double *o, const double *d, double best, double &tn) {
  double t0 = -1e300, t1 = 1e300;
  for (int k = 0; k < 3; k++) {
    if (d[k] == 0.0) {
      if (o[k] < b.lo[k] || o[k] > b.hi[k]) return false;
      continue;
    }
    double a = (b.lo[k] - o[k]) / d[k], c = (b.hi[k] - o[k]) / d[k];
    if (a > c) std::swap(a, c);
    t0 = std::max(t0, a);
    t1 = std::min(t1, c);
  }
  tn = t0;
  return t0 <= t1 && t1 >= 0.0 && t0 <= best;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s tris.bin n_rays seed\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { printf("cannot open %s\n", argv[1]); return 1; }
  fseek(f, 0, SEEK_END);
  const long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  const int n = (int)(sz / 36);
  std::vector<float> T(9 * (size_t)n);
  if (n > 0 && fread(T.data(), 1, (size_t)sz, f) != (size_t)sz) { printf("short read\n"); return 1; }
  fclose(f);
  const int n_rays = atoi(argv[2]);
  srand((unsigned)atoi(argv[3]));

  std::vector<BvhNode> nodes;
  std::vector<int> perm;
  char msg[256] = {0};
  if (!sah_build_triangles(T.data(), n, nodes, perm, msg, sizeof msg)) {
    printf("build failed: %s\n", msg);
    return 1;
  }
  if ((int)perm.size() != n || (int)nodes.size() != (n > 1 ? n - 1 : 0)) {
    printf("sizes: perm %zu nodes %zu for n %d\n", perm.size(), nodes.size(), n);
    return 1;
  }
  std::vector<char> seen_p((size_t)n, 0);
  for (int i = 0; i < n; i++) {
    if (perm[i] < 0 || perm[i] >= n || seen_p[(size_t)perm[i]]) { printf("perm not a permutation\n"); return 1; }
    seen_p[(size_t)perm[i]] = 1;
  }
  auto tri_box = [&](int sorted) {
    const float *v = &T[9 * (size_t)perm[sorted]];
    Box b;
    for (int k = 0; k < 3; k++) {
      b.lo[k] = std::min(std::min(v[k], v[3 + k]), v[6 + k]);
      b.hi[k] = std::max(std::max(v[k], v[3 + k]), v[6 + k]);
    }
    return b;
  };
  // structure: reach every node once, boxes contain subtrees, depth
  int max_depth = 0;
  if (n > 1) {
    std::vector<char> seen_n(nodes.size(), 0), seen_l((size_t)n, 0);
    struct Item { int node, depth; };
    std::vector<Item> st{{0, 0}};
    // subtree box check: the child box must contain every triangle below it
    std::vector<std::vector<int>> below(nodes.size());
    std::vector<int> order;
    while (!st.empty()) {
      Item it = st.back();
      st.pop_back();
      if (it.node < 0 || it.node >= (int)nodes.size() || seen_n[(size_t)it.node]) {
        printf("node %d reached twice or out of range\n", it.node);
        return 1;
      }
      seen_n[(size_t)it.node] = 1;
      order.push_back(it.node);
      max_depth = std::max(max_depth, it.depth + 1);
      const int ch[2] = {nodes[(size_t)it.node].d.x, nodes[(size_t)it.node].d.y};
      for (int c = 0; c < 2; c++) {
        if (ch[c] < 0) {
          const int l = ~ch[c];
          if (l >= n || seen_l[(size_t)l]) { printf("leaf %d repeated\n", l); return 1; }
          seen_l[(size_t)l] = 1;
          if (!contains(child_box(nodes[(size_t)it.node], c), tri_box(l))) {
            printf("leaf box of node %d child %d does not contain its triangle\n", it.node, c);
            return 1;
          }
        } else {
          st.push_back({ch[c], it.depth + 1});
        }
      }
    }
    for (size_t i = 0; i < nodes.size(); i++)
      if (!seen_n[i]) { printf("node %zu unreachable\n", i); return 1; }
    // containment of internal children: every triangle under child c lies in its box
    std::vector<std::vector<int>> leaves(nodes.size());
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
      const BvhNode &nd = nodes[(size_t)*it];
      const int ch[2] = {nd.d.x, nd.d.y};
      for (int c = 0; c < 2; c++) {
        std::vector<int> sub;
        if (ch[c] < 0) sub.push_back(~ch[c]);
        else sub = leaves[(size_t)ch[c]];
        const Box cb = child_box(nd, c);
        for (int l : sub)
          if (!contains(cb, tri_box(l))) {
            printf("child box %d of node %d misses triangle %d\n", c, *it, l);
            return 1;
          }
        leaves[(size_t)*it].insert(leaves[(size_t)*it].end(), sub.begin(), sub.end());
      }
      if (*it != 0) {
        for (int c = 0; c < 2; c++) if (ch[c] >= 0) { leaves[(size_t)ch[c]].clear(); leaves[(size_t)ch[c]].shrink_to_fit(); }
      }
    }
    if (max_depth > 62) { printf("depth %d exceeds the traversal stack\n", max_depth); return 1; }
  }
  // closest hits: tree traversal vs brute force
  float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
  for (int i = 0; i < 3 * n; i++)
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], T[3 * (size_t)i + k]);
      hi[k] = std::max(hi[k], T[3 * (size_t)i + k]);
    }
  for (int r = 0; r < n_rays && n > 0; r++) {
    double o[3], d[3];
    for (int k = 0; k < 3; k++) o[k] = lo[k] + (hi[k] - lo[k]) * (rand() / (double)RAND_MAX);
    const double z = 2.0 * (rand() / (double)RAND_MAX) - 1.0,
                 ph = 6.283185307179586 * (rand() / (double)RAND_MAX), s = std::sqrt(1.0 - z * z);
    d[0] = s * std::cos(ph); d[1] = s * std::sin(ph); d[2] = z;
    if (r % 7 == 0) { d[0] = 0.0; d[1] = 0.0; d[2] = (r % 2) ? 1.0 : -1.0; }  // axis-parallel
    double bt = 1e300;
    int bp = -1;
    for (int i = 0; i < n; i++) {
      const double t = tri_t(&T[9 * (size_t)i], o, d);
      if (t > 0.0 && (t < bt || (t == bt && i < bp))) { bt = t; bp = i; }
    }
    double tt = 1e300;
    int tp = -1;
    auto test_leaf = [&](int l) {
      const int orig = perm[l];
      const double t = tri_t(&T[9 * (size_t)orig], o, d);
      if (t > 0.0 && (t < tt || (t == tt && orig < tp))) { tt = t; tp = orig; }
    };
    if (n == 1) {
      test_leaf(0);
    } else {
      std::vector<std::pair<int, double>> st;
      int node = 0;
      while (true) {
        const BvhNode &nd = nodes[(size_t)node];
        double t0, t1;
        bool h0 = slab(child_box(nd, 0), o, d, tt, t0), h1 = slab(child_box(nd, 1), o, d, tt, t1);
        if (h0 && nd.d.x < 0) { test_leaf(~nd.d.x); h0 = false; }
        if (h1 && nd.d.y < 0) { test_leaf(~nd.d.y); h1 = false; }
        if (h0 && h1) {
          int nr = nd.d.x, fr = nd.d.y;
          double tf = t1;
          if (t1 < t0) { nr = nd.d.y; fr = nd.d.x; tf = t0; }
          st.push_back({fr, tf});
          node = nr;
        } else if (h0) {
          node = nd.d.x;
        } else if (h1) {
          node = nd.d.y;
        } else {
          bool found = false;
          while (!st.empty()) {
            auto e = st.back();
            st.pop_back();
            if (e.second <= tt) { node = e.first; found = true; break; }
          }
          if (!found) break;
        }
      }
    }
    if (tp != bp || (bp >= 0 && tt != bt)) {
      printf("ray %d: tree hit %d at %.17g, brute force %d at %.17g\n", r, tp, tt, bp, bt);
      return 1;
    }
  }
  printf("ok %zu %d\n", nodes.size(), max_depth);
  return 0;
}
