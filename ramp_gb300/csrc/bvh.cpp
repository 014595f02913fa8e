/*
 * bvh.cpp — host construction of the bounding volume hierarchy used by the
 * GMesh kernel (binned surface-area heuristic, 16 bins per axis, leaves of
 * at most 4 triangles, depth capped so a 64-entry traversal stack always
 * suffices), stored with each inner node holding its children's boxes.
 * Output layout is described in mesh.cuh.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "bvh.h"

namespace {

struct Box {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
  }
  void grow(const float* p) {
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
  }
  void grow(const Box& b) {
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
  }
  double area() const {
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = std::max(0.0, (double)hi[k] - (double)lo[k]);
    return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
  }
};

struct Builder {
  const float* pts;
  std::vector<Box> tbox;
  std::vector<float> cen;      /* 3 per triangle */
  std::vector<int> order;
  std::vector<float> nodes;    /* 8 floats per node */

  int new_node() {
    nodes.resize(nodes.size() + 8, 0.0f);
    return (int)(nodes.size() / 8) - 1;
  }

  static float as_float(int v) { float f; std::memcpy(&f, &v, 4); return f; }

  void set_node(int ni, const Box& b, int wa, int wb) {
    float* o = &nodes[8 * (size_t)ni];
    /* inflate so float rounding in the device slab test never culls a
       triangle the exact test accepts */
    for (int k = 0; k < 3; ++k) {
      float ext = b.hi[k] - b.lo[k];
      float mag = std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k]));
      float pad = 1e-4f * ext + 1e-6f * mag + 1e-7f;
      o[k] = b.lo[k] - pad;
      o[4 + k] = b.hi[k] + pad;
    }
    o[3] = as_float(wa);
    o[7] = as_float(wb);
  }

  void build(int ni, int begin, int end, int depth) {
    Box b, cb;
    b.reset(); cb.reset();
    for (int i = begin; i < end; ++i) {
      b.grow(tbox[order[i]]);
      cb.grow(&cen[3 * (size_t)order[i]]);
    }
    int count = end - begin;
    if (count <= 4 || depth >= 48) {
      set_node(ni, b, begin, -count);
      return;
    }
    const int NB = 16;
    double best = INFINITY;
    int best_axis = -1, best_split = -1;
    for (int ax = 0; ax < 3; ++ax) {
      float lo = cb.lo[ax], hi = cb.hi[ax];
      if (!(hi > lo)) continue;
      Box bins[NB];
      int cnt[NB] = {0};
      for (int k = 0; k < NB; ++k) bins[k].reset();
      float scale = NB / (hi - lo);
      for (int i = begin; i < end; ++i) {
        int t = order[i];
        int k = std::min(NB - 1, (int)((cen[3 * (size_t)t + ax] - lo) * scale));
        cnt[k]++;
        bins[k].grow(tbox[t]);
      }
      Box lb[NB], rb[NB];
      int lc[NB], rc[NB];
      Box acc; acc.reset(); int n = 0;
      for (int k = 0; k < NB; ++k) { acc.grow(bins[k]); n += cnt[k]; lb[k] = acc; lc[k] = n; }
      acc.reset(); n = 0;
      for (int k = NB - 1; k >= 0; --k) { acc.grow(bins[k]); n += cnt[k]; rb[k] = acc; rc[k] = n; }
      for (int k = 0; k < NB - 1; ++k) {
        if (lc[k] == 0 || rc[k + 1] == 0) continue;
        double cost = lb[k].area() * lc[k] + rb[k + 1].area() * rc[k + 1];
        if (cost < best) { best = cost; best_axis = ax; best_split = k; }
      }
    }
    int mid;
    if (best_axis < 0) {
      mid = begin + count / 2;
    } else {
      float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
      float scale = NB / (hi - lo);
      int* p = std::partition(&order[begin], &order[begin] + count, [&](int t) {
        int k = std::min(NB - 1, (int)((cen[3 * (size_t)t + best_axis] - lo) * scale));
        return k <= best_split;
      });
      mid = (int)(p - &order[0]);
      if (mid == begin || mid == end) mid = begin + count / 2;
    }
    int l = new_node();
    int r = new_node();
    set_node(ni, b, l, r);
    build(l, begin, mid, depth + 1);
    build(r, mid, end, depth + 1);
  }
};

}  // namespace

int ramp_bvh_build(const float* pts, int64_t n_tri, std::vector<float>& nodes,
                   std::vector<float>& tris) {
  if (n_tri <= 0) return -1;
  Builder B;
  B.pts = pts;
  B.tbox.resize((size_t)n_tri);
  B.cen.resize(3 * (size_t)n_tri);
  B.order.resize((size_t)n_tri);
  for (int64_t t = 0; t < n_tri; ++t) {
    const float* p = pts + 9 * t;
    B.tbox[t].reset();
    B.tbox[t].grow(p); B.tbox[t].grow(p + 3); B.tbox[t].grow(p + 6);
    for (int k = 0; k < 3; ++k) B.cen[3 * t + k] = (p[k] + p[3 + k] + p[6 + k]) / 3.0f;
    B.order[t] = (int)t;
  }
  int root = B.new_node();
  B.build(root, 0, (int)n_tri, 0);
  /* store each inner node as its two children's boxes and references, so
     one 64-byte read tests both children: per child (lo.xyz, a),
     (hi.xyz, b) with b >= 1 a leaf of b triangles from a, b == 0 the inner
     node a, b == -1 no child (only beside a root that is a leaf) */
  const std::vector<float>& bn = B.nodes;
  const size_t n_old = bn.size() / 8;
  std::vector<int> newid(n_old, -1);
  int n_inner = 0;
  for (size_t i = 0; i < n_old; ++i) {
    int wb;
    std::memcpy(&wb, &bn[8 * i + 7], 4);
    if (wb >= 0) newid[i] = n_inner++;
  }
  auto child = [&](float* o, size_t c) {
    int wa, wb;
    std::memcpy(&wa, &bn[8 * c + 3], 4);
    std::memcpy(&wb, &bn[8 * c + 7], 4);
    for (int k = 0; k < 3; ++k) { o[k] = bn[8 * c + k]; o[4 + k] = bn[8 * c + 4 + k]; }
    const int a = wb >= 0 ? newid[c] : wa, b = wb >= 0 ? 0 : -wb;
    std::memcpy(&o[3], &a, 4);
    std::memcpy(&o[7], &b, 4);
  };
  nodes.assign(16 * (size_t)std::max(n_inner, 1), 0.0f);
  if (n_inner == 0) {            /* the root is a leaf: one node, one child */
    child(&nodes[0], 0);
    const int none = -1;
    std::memcpy(&nodes[15], &none, 4);
  } else {
    for (size_t i = 0; i < n_old; ++i) {
      if (newid[i] < 0) continue;
      int wa, wb;
      std::memcpy(&wa, &bn[8 * i + 3], 4);
      std::memcpy(&wb, &bn[8 * i + 7], 4);
      float* o = &nodes[16 * (size_t)newid[i]];
      child(o, (size_t)wa);
      child(o + 8, (size_t)wb);
    }
  }
  tris.assign(12 * (size_t)n_tri, 0.0f);
  for (int64_t i = 0; i < n_tri; ++i) {
    const float* p = pts + 9 * (size_t)B.order[i];
    float* o = &tris[12 * (size_t)i];
    o[0] = p[0]; o[1] = p[1]; o[2] = p[2];
    o[4] = p[3]; o[5] = p[4]; o[6] = p[5];
    o[8] = p[6]; o[9] = p[7]; o[10] = p[8];
  }
  return 0;
}
