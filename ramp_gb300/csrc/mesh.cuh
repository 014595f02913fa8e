/*
 * mesh.cuh — GMesh intersection (mcramp/geom/mesh.cl:3-129) through a
 * bounding volume hierarchy.
 *
 * The reference tests every triangle for every ray.  Its result does not
 * depend on the order in which triangles are visited: the entering and
 * exiting records keep the smallest t (ties give identical records, the
 * point being pos + vel*t), the crossing count is a sum, and the chord
 * (for SAttenuate) is built from the sorted crossings.  So a traversal that
 * reaches every triangle the ray can hit returns the reference's record.
 * For SAttenuate the crossings (t, sign)
 * are collected, sorted, and each entry is paired with the next exit
 * (repeated entries or exits, which a ray through an edge shared by two
 * faces can produce, are ignored); the ray is taken to start outside.
 * Node boxes are inflated at build time
 * so that float rounding in the slab test never culls a triangle that the
 * Moller-Trumbore test accepts; without interior parity or chord sums,
 * nodes that start beyond both current records are pruned.
 *
 * Node layout: 2 float4 per node, (min.xyz, a) (max.xyz, b); b >= 0: inner
 * node with children a and b; b < 0: leaf with triangles [a, a - b).
 * Triangle layout: 3 float4, v0, e1 = v1 - v0, e2 = v2 - v0 (host float
 * subtraction, the same values the reference computes per test).
 */
#ifndef RAMP_MESH_CUH
#define RAMP_MESH_CUH

#define RAMP_BVH_STACK 64
#define RAMP_MESH_MAX_HITS 16

DI float chord_from_hits(float* t, int* sg, int nh) {
  for (int a = 1; a < nh; ++a) {
    float tv = t[a]; int sv = sg[a]; int b = a - 1;
    while (b >= 0 && (t[b] > tv || (t[b] == tv && sg[b] > sv))) { t[b + 1] = t[b]; sg[b + 1] = sg[b]; --b; }
    t[b + 1] = tv; sg[b + 1] = sv;
  }
  double chord = 0.0, t_in = 0.0;
  bool inside = false;
  for (int a = 0; a < nh; ++a) {
    if (sg[a] < 0 && !inside) { inside = true; t_in = t[a]; }
    else if (sg[a] > 0 && inside) { inside = false; chord += (double)t[a] - t_in; }
  }
  return (float)chord;
}

DI bool g_mesh(const CompDev& c, Nt& n, Is& s, StatusDev* st) {
  V3 pos = npos(n), vel = nvel(n);
  /* bounding box of the whole mesh, mesh.cl:22-40 */
  V3 ll = v3(c.gp[0], c.gp[2], c.gp[4]), ur = v3(c.gp[1], c.gp[3], c.gp[5]);
  V3 dA = sub(ll, pos), dB = sub(ur, pos);
  float t1 = dA.x / vel.x, t2 = dB.x / vel.x, t3 = dA.y / vel.y;
  float t4 = dB.y / vel.y, t5 = dA.z / vel.z, t6 = dB.z / vel.z;
  float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
  float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
  if (tmax < 0.0f || tmin > tmax) return false;

  const float eps = 0.000000001f;
  const bool need_all = (c.gi[0] == 1) || (c.scat == RAMP_S_ATTENUATE);
  uint32_t num_intersections = 0;
  float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f, o3 = 1e8f, o4 = 0.0f, o5 = 0.0f, o6 = 0.0f, o7 = 1e8f;
  const bool want_chord = (c.scat == RAMP_S_ATTENUATE);
  float ht[RAMP_MESH_MAX_HITS];
  int hs[RAMP_MESH_MAX_HITS];
  int nh = 0;
  const float ix = 1.0f / vel.x, iy = 1.0f / vel.y, iz = 1.0f / vel.z;
  const float4* __restrict__ nodes = c.bvh_nodes;
  const float4* __restrict__ tris = c.bvh_tris;
  int stack[RAMP_BVH_STACK];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    int ni = stack[--sp];
    float4 a = __ldg(nodes + 2 * ni), b = __ldg(nodes + 2 * ni + 1);
    float tx0 = (a.x - pos.x) * ix, tx1 = (b.x - pos.x) * ix;
    float ty0 = (a.y - pos.y) * iy, ty1 = (b.y - pos.y) * iy;
    float tz0 = (a.z - pos.z) * iz, tz1 = (b.z - pos.z) * iz;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    if (tn > tf || tf < -1e-6f) continue;
    if (!need_all && tn > fmaxf(o3, o7)) continue;
    int wa = __float_as_int(a.w), wb = __float_as_int(b.w);
    if (wb >= 0) {
      if (sp + 2 > RAMP_BVH_STACK) { raise_flag(st, RAMP_F_BVH_STACK); return false; }
      stack[sp++] = wa;
      stack[sp++] = wb;
      continue;
    }
    for (int k = wa; k < wa - wb; ++k) {
      float4 q0 = __ldg(tris + 3 * k), q1 = __ldg(tris + 3 * k + 1), q2 = __ldg(tris + 3 * k + 2);
      V3 v0 = v3(q0.x, q0.y, q0.z), e1 = v3(q1.x, q1.y, q1.z), e2 = v3(q2.x, q2.y, q2.z);
      V3 h = cross(vel, e2);
      float aa = dot(e1, h);
      if (fabsf(aa) < eps) continue;
      float f = 1.0f / aa;
      V3 sv = sub(pos, v0);
      float u = f * dot(sv, h);
      if (u < 0.0f || u > 1.0f) continue;
      V3 qv = cross(sv, e1);
      float v = f * dot(vel, qv);
      if (v < 0.0f || u + v > 1.0f) continue;
      float t = f * dot(e2, qv);
      if (t > eps) num_intersections++;
      V3 nrm = cross(e1, e2);
      float nv = dot(nrm, vel);
      if ((t > eps) && (t < o3) && (nv < 0)) {
        o0 = pos.x + vel.x * t; o1 = pos.y + vel.y * t; o2 = pos.z + vel.z * t; o3 = t;
      }
      if ((t > eps) && (t < o7) && (nv > 0)) {
        o4 = pos.x + vel.x * t; o5 = pos.y + vel.y * t; o6 = pos.z + vel.z * t; o7 = t;
      }
      if (want_chord && t > eps && nv != 0) {
        if (nh < RAMP_MESH_MAX_HITS) { ht[nh] = t; hs[nh] = nv > 0 ? 1 : -1; ++nh; }
        else raise_flag(st, RAMP_F_BVH_STACK);
      }
    }
  }
  if ((c.gi[0] == 1) && (num_intersections % 2 == 1)) {
    o4 = o0; o5 = o1; o6 = o2; o7 = o3;
  } else if ((c.gi[0] == 1) && (num_intersections % 2 == 0)) {
    return false;
  }
  if (o3 < s.t1) {
    s.x1 = o0; s.y1 = o1; s.z1 = o2; s.t1 = o3;
    s.x2 = o4; s.y2 = o5; s.z2 = o6; s.t2 = o7;
    if (want_chord) { n.sd = chord_from_hits(ht, hs, nh); n.wr |= WR_SD; }
    return true;
  }
  return false;
}

#endif /* RAMP_MESH_CUH */
