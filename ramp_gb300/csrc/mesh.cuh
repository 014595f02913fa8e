/*
 * mesh.cuh — GMesh intersection (mcramp/geom/mesh.cl:3-129) through a
 * bounding volume hierarchy.
 *
 * The reference tests every triangle for every ray (Moller-Trumbore).  Its
 * record does not depend on the order in which triangles are visited: the
 * entering and exiting hits keep the smallest t (ties give identical
 * records, the point being pos + vel*t) and the crossing count is a sum.
 * So a traversal that reaches every triangle the ray can hit returns the
 * reference's record.  Node boxes are inflated at build time so that float
 * rounding in the slab test never culls a triangle the exact test accepts;
 * without interior parity or a chord, nodes that start beyond both current
 * records are pruned.
 *
 * For SAttenuate the chord is the sum over watertight crossings (Woop,
 * Benthin, Wald, JCGT 2013) of +t leaving / -t entering, accumulated in
 * double: exact for the few dozen crossings of one ray, so independent of
 * the visiting order; clamped at 0.
 *
 * Node layout: each inner node is 4 float4, its two children's boxes and
 * references, per child (min.xyz, a) (max.xyz, b): b >= 1 a leaf with
 * triangles [a, a + b), b == 0 the inner node a, b == -1 no child; node 0
 * is the root.  One 64-byte read tests both children; leaves are tested at
 * once, and the traversal continues into the nearer inner child.
 * Triangle layout: 3 float4, the vertices v0, v1, v2; edges are formed as
 * the reference forms them (v1 - v0, v2 - v0 in float).
 */
#ifndef RAMP_MESH_CUH
#define RAMP_MESH_CUH

#define RAMP_BVH_STACK 64

struct Shear { int kx, ky, kz; float Sx, Sy, Sz; };

DI float comp3(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

DI Shear make_shear(V3 d) {
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  Shear S;
  S.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  S.kx = (S.kz + 1) % 3; S.ky = (S.kx + 1) % 3;
  if (comp3(d, S.kz) < 0.0f) { int t = S.kx; S.kx = S.ky; S.ky = t; }
  S.Sx = comp3(d, S.kx) / comp3(d, S.kz);
  S.Sy = comp3(d, S.ky) / comp3(d, S.kz);
  S.Sz = 1.0f / comp3(d, S.kz);
  return S;
}

/* watertight crossing parameter t, NaN when the ray misses the face */
DI float watertight_t(const Shear& S, V3 org, V3 v0, V3 v1, V3 v2) {
  V3 A = sub(v0, org), B = sub(v1, org), C = sub(v2, org);
  float Akz = comp3(A, S.kz), Bkz = comp3(B, S.kz), Ckz = comp3(C, S.kz);
  float Ax = comp3(A, S.kx) - S.Sx * Akz, Ay = comp3(A, S.ky) - S.Sy * Akz;
  float Bx = comp3(B, S.kx) - S.Sx * Bkz, By = comp3(B, S.ky) - S.Sy * Bkz;
  float Cx = comp3(C, S.kx) - S.Sx * Ckz, Cy = comp3(C, S.ky) - S.Sy * Ckz;
  float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return __int_as_float(0x7fc00000);
  float det = U + V + W;
  if (det == 0.0f) return __int_as_float(0x7fc00000);
  float T = U * (S.Sz * Akz) + V * (S.Sz * Bkz) + W * (S.Sz * Ckz);
  return T / det;
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
  Shear S;
  if (want_chord) S = make_shear(vel);
  double chord = 0.0;
  const float ix = 1.0f / vel.x, iy = 1.0f / vel.y, iz = 1.0f / vel.z;
  const float4* __restrict__ nodes = c.bvh_nodes;
  const float4* __restrict__ tris = c.bvh_tris;
  int stack[RAMP_BVH_STACK];
  int sp = 0;
  int node = 0;
  for (;;) {
    const float4* q = nodes + 4 * node;
    const float4 a0 = __ldg(q), b0 = __ldg(q + 1), a1 = __ldg(q + 2), b1 = __ldg(q + 3);
    const int r0 = __float_as_int(a0.w), c0 = __float_as_int(b0.w);
    const int r1 = __float_as_int(a1.w), c1 = __float_as_int(b1.w);
    float tn0 = 0.0f, tn1 = 0.0f;
    bool h0 = false, h1 = false;
    if (c0 >= 0) {
      float tx0 = (a0.x - pos.x) * ix, tx1 = (b0.x - pos.x) * ix;
      float ty0 = (a0.y - pos.y) * iy, ty1 = (b0.y - pos.y) * iy;
      float tz0 = (a0.z - pos.z) * iz, tz1 = (b0.z - pos.z) * iz;
      tn0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
      float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
      h0 = !(tn0 > tf || tf < -1e-6f) && (need_all || !(tn0 > fmaxf(o3, o7)));
    }
    if (c1 >= 0) {
      float tx0 = (a1.x - pos.x) * ix, tx1 = (b1.x - pos.x) * ix;
      float ty0 = (a1.y - pos.y) * iy, ty1 = (b1.y - pos.y) * iy;
      float tz0 = (a1.z - pos.z) * iz, tz1 = (b1.z - pos.z) * iz;
      tn1 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
      float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
      h1 = !(tn1 > tf || tf < -1e-6f) && (need_all || !(tn1 > fmaxf(o3, o7)));
    }
    /* the triangles of the leaf children that were hit, as one range */
    const int n0 = (h0 && c0 > 0) ? c0 : 0, n1 = (h1 && c1 > 0) ? c1 : 0;
    for (int j = 0; j < n0 + n1; ++j) {
      const int k = j < n0 ? r0 + j : r1 + (j - n0);
      float4 q0 = __ldg(tris + 3 * k), q1 = __ldg(tris + 3 * k + 1), q2 = __ldg(tris + 3 * k + 2);
      V3 v0 = v3(q0.x, q0.y, q0.z), v1 = v3(q1.x, q1.y, q1.z), v2 = v3(q2.x, q2.y, q2.z);
      V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
      if (want_chord) {
        float tw = watertight_t(S, pos, v0, v1, v2);
        if (tw > eps) {
          float nvw = dot(cross(e1, e2), vel);
          if (nvw > 0) chord += (double)tw;
          else if (nvw < 0) chord -= (double)tw;
        }
      }
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
    }
    /* inner children: continue into the nearer, keep the other */
    const bool i0 = h0 && c0 == 0, i1 = h1 && c1 == 0;
    if (i0 && i1) {
      if (sp + 1 > RAMP_BVH_STACK) { raise_flag(st, RAMP_F_BVH_STACK); return false; }
      const bool first0 = !(tn1 < tn0);
      stack[sp++] = first0 ? r1 : r0;
      node = first0 ? r0 : r1;
    } else if (i0) {
      node = r0;
    } else if (i1) {
      node = r1;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
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
    if (want_chord) { n.sd = chord > 0.0 ? (float)chord : 0.0f; n.wr |= WR_SD; }
    return true;
  }
  return false;
}

#endif /* RAMP_MESH_CUH */
