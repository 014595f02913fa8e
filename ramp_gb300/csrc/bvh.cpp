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
#include "../../include/ramp.h"

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

/* Memory the GMesh walk reads for a set of rays when it needs every
 * crossing (interior parity or a chord, as SAttenuate): every inner node
 * whose box the ray meets is read once (64 bytes: both children's boxes)
 * and every triangle of a leaf whose box it meets is read once (48 bytes).
 * The walk order does not change these counts.  The slab tests are the
 * device's (mesh.cuh), in float.  rays: 6 floats each (position, velocity)
 * in the mesh's frame; out[0] inner nodes read, out[1] triangles read,
 * out[2] rays that meet the mesh's bounding box. */
extern "C" int ramp_bvh_walk_counts(const float* pts, int64_t n_tri, const float* rays,
                                    int64_t n_rays, int64_t* out) {
  if (!pts || !rays || !out || n_tri <= 0 || n_rays < 0) return -1;
  std::vector<float> nodes, tris;
  if (ramp_bvh_build(pts, n_tri, nodes, tris) != 0) return -1;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < 3 * n_tri; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], pts[3 * i + k]);
      hi[k] = std::max(hi[k], pts[3 * i + k]);
    }
  int64_t n_nodes = 0, n_tris = 0, n_in = 0;
  std::vector<int> stack;
  for (int64_t r = 0; r < n_rays; ++r) {
    const float* p = rays + 6 * r;
    const float* v = p + 3;
    float tmin = -INFINITY, tmax = INFINITY;
    for (int k = 0; k < 3; ++k) {
      const float t1 = (lo[k] - p[k]) / v[k], t2 = (hi[k] - p[k]) / v[k];
      tmin = std::max(tmin, std::min(t1, t2));
      tmax = std::min(tmax, std::max(t1, t2));
    }
    if (tmax < 0.0f || tmin > tmax) continue;
    ++n_in;
    const float inv[3] = {1.0f / v[0], 1.0f / v[1], 1.0f / v[2]};
    stack.assign(1, 0);
    while (!stack.empty()) {
      const int nd = stack.back();
      stack.pop_back();
      ++n_nodes;
      const float* q = &nodes[16 * (size_t)nd];
      for (int c = 0; c < 2; ++c) {
        const float* b = q + 8 * c;
        int a, cnt;
        std::memcpy(&a, &b[3], 4);
        std::memcpy(&cnt, &b[7], 4);
        if (cnt < 0) continue;
        float tn = -INFINITY, tf = INFINITY;
        for (int k = 0; k < 3; ++k) {
          const float t0 = (b[k] - p[k]) * inv[k], t1 = (b[4 + k] - p[k]) * inv[k];
          tn = std::max(tn, std::min(t0, t1));
          tf = std::min(tf, std::max(t0, t1));
        }
        if (tn > tf || tf < -1e-6f) continue;
        if (cnt > 0) n_tris += cnt;
        else stack.push_back(a);
      }
    }
  }
  out[0] = n_nodes;
  out[1] = n_tris;
  out[2] = n_in;
  return 0;
}
