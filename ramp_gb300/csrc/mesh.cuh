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
 * is the root.  One 64-byte read tests both children; the traversal
 * continues into the nearer inner child.  When both children are leaves
 * the second's triangles follow the first's (a1 = a0 + b0), so the hit
 * leaves of a node are one triangle range.
 * Triangle layout: 3 float4, the vertices v0, v1, v2; edges are formed as
 * the reference forms them (v1 - v0, v2 - v0 in float).
 */
#ifndef RAMP_MESH_CUH
#define RAMP_MESH_CUH

#define RAMP_BVH_STACK 64
/* stack entries a walk kernel keeps per thread in shared memory (the rest
 * go to the thread's local array) */
#define RAMP_BVH_SSTACK 16

/* the ray's shear: axis indices kx | ky << 2 | kz << 4 in one word (fewer
 * live registers in the walk), and the three shear factors */
struct Shear { int k; float Sx, Sy, Sz; };
DI int shear_kx(const Shear& S) { return S.k & 3; }
DI int shear_ky(const Shear& S) { return (S.k >> 2) & 3; }
DI int shear_kz(const Shear& S) { return S.k >> 4; }

DI float comp3(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

DI Shear make_shear(V3 d) {
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  Shear S;
  const int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (comp3(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
  S.k = kx | (ky << 2) | (kz << 4);
  S.Sx = comp3(d, kx) / comp3(d, kz);
  S.Sy = comp3(d, ky) / comp3(d, kz);
  S.Sz = 1.0f / comp3(d, kz);
  return S;
}

/* watertight crossing parameter t, NaN when the ray misses the face */
DI float watertight_t(const Shear& S, V3 org, V3 v0, V3 v1, V3 v2) {
  V3 A = sub(v0, org), B = sub(v1, org), C = sub(v2, org);
  const int kx = shear_kx(S), ky = shear_ky(S), kz = shear_kz(S);
  float Akz = comp3(A, kz), Bkz = comp3(B, kz), Ckz = comp3(C, kz);
  float Ax = comp3(A, kx) - S.Sx * Akz, Ay = comp3(A, ky) - S.Sy * Akz;
  float Bx = comp3(B, kx) - S.Sx * Bkz, By = comp3(B, ky) - S.Sy * Bkz;
  float Cx = comp3(C, kx) - S.Sx * Ckz, Cy = comp3(C, ky) - S.Sy * Ckz;
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

/* The walk of one ray through the hierarchy, resumable (mesh_begin, then
 * mesh_step until it returns 0 or -1, then mesh_end): g_mesh runs it to the
 * end for one neutron.  The same walk also comes as its two kinds of work,
 * for kernels that interleave the walks of many rays on one lane and pick
 * per pass which kind the lanes of a warp run: mesh_visit tests one inner
 * node's children and leaves the triangles of its hit leaf children as the
 * range [tb, te) (the triangles of sibling leaves are adjacent, so one range
 * covers both); mesh_tri tests one triangle of that range.  Such a walk is
 * over when the range is empty and no node is left (mesh_walk_over). */
/* per component: the walk needs every crossing (interior parity or a
 * chord) / accumulates SAttenuate's chord */
DI bool mesh_all(const CompDev& c) { return (c.gi[0] == 1) || (c.scat == RAMP_S_ATTENUATE); }
DI bool mesh_chord(const CompDev& c) { return c.scat == RAMP_S_ATTENUATE; }

struct MeshWalk {
  V3 pos, vel;
  float ix, iy, iz;
  float o3, o7;          /* t of the entering and exiting records (1e8: none) */
  double chord;
  uint32_t num_intersections;
  int sp, node, tb, te;
  Shear S;
  int stack[RAMP_BVH_STACK];
};

/* what a finished walk leaves for mesh_end */
struct MeshRec { float o3, o7; double chord; uint32_t num_intersections; };

DI MeshRec mesh_rec(const MeshWalk& w) {
  MeshRec r;
  r.o3 = w.o3; r.o7 = w.o7; r.chord = w.chord; r.num_intersections = w.num_intersections;
  return r;
}

/* bounding box of the whole mesh (mesh.cl:22-40); false: the ray misses it
 * and the intersection is false */
DI bool mesh_begin(const CompDev& c, const Nt& n, MeshWalk& w) {
  V3 pos = npos(n), vel = nvel(n);
  V3 ll = v3(c.gp[0], c.gp[2], c.gp[4]), ur = v3(c.gp[1], c.gp[3], c.gp[5]);
  V3 dA = sub(ll, pos), dB = sub(ur, pos);
  float t1 = dA.x / vel.x, t2 = dB.x / vel.x, t3 = dA.y / vel.y;
  float t4 = dB.y / vel.y, t5 = dA.z / vel.z, t6 = dB.z / vel.z;
  float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
  float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
  if (tmax < 0.0f || tmin > tmax) return false;
  w.pos = pos;
  w.vel = vel;
  w.num_intersections = 0;
  w.o3 = 1e8f;
  w.o7 = 1e8f;
  if (mesh_chord(c)) w.S = make_shear(vel);
  w.chord = 0.0;
  w.ix = 1.0f / vel.x; w.iy = 1.0f / vel.y; w.iz = 1.0f / vel.z;
  w.sp = 0;
  w.node = 0;
  w.tb = 0; w.te = 0;
  return true;
}

/* triangle k (mesh.cl:48-112): the chord crossing, then Moller-Trumbore and
 * the entering and exiting records */
DI void mesh_tri(const CompDev& c, MeshWalk& w, int k) {
  const float eps = 0.000000001f;
  const V3 pos = w.pos, vel = w.vel;
  const float4* __restrict__ tris = c.bvh_tris;
  float4 q0 = __ldg(tris + 3 * k), q1 = __ldg(tris + 3 * k + 1), q2 = __ldg(tris + 3 * k + 2);
  V3 v0 = v3(q0.x, q0.y, q0.z), v1 = v3(q1.x, q1.y, q1.z), v2 = v3(q2.x, q2.y, q2.z);
  V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  if (mesh_chord(c)) {
    float tw = watertight_t(w.S, pos, v0, v1, v2);
    if (tw > eps) {
      float nvw = dot(cross(e1, e2), vel);
      if (nvw > 0) w.chord += (double)tw;
      else if (nvw < 0) w.chord -= (double)tw;
    }
  }
  V3 h = cross(vel, e2);
  float aa = dot(e1, h);
  if (fabsf(aa) < eps) return;
  float f = 1.0f / aa;
  V3 sv = sub(pos, v0);
  float u = f * dot(sv, h);
  if (u < 0.0f || u > 1.0f) return;
  V3 qv = cross(sv, e1);
  float v = f * dot(vel, qv);
  if (v < 0.0f || u + v > 1.0f) return;
  float t = f * dot(e2, qv);
  if (t > eps) w.num_intersections++;
  V3 nrm = cross(e1, e2);
  float nv = dot(nrm, vel);
  /* the points pos + vel * t of the records are formed at the end */
  if ((t > eps) && (t < w.o3) && (nv < 0)) w.o3 = t;
  if ((t > eps) && (t < w.o7) && (nv > 0)) w.o7 = t;
}

/* the slab tests of inner node w.node's two children */
struct MeshKids { int r0, c0, r1, c1; float tn0, tn1; bool h0, h1; };

DI MeshKids mesh_kids(const CompDev& c, const MeshWalk& w) {
  const bool all = mesh_all(c);
  const V3 pos = w.pos;
  const float ix = w.ix, iy = w.iy, iz = w.iz;
  const float4* q = c.bvh_nodes + 4 * w.node;
  const float4 a0 = __ldg(q), b0 = __ldg(q + 1), a1 = __ldg(q + 2), b1 = __ldg(q + 3);
  MeshKids K;
  K.r0 = __float_as_int(a0.w); K.c0 = __float_as_int(b0.w);
  K.r1 = __float_as_int(a1.w); K.c1 = __float_as_int(b1.w);
  K.tn0 = 0.0f; K.tn1 = 0.0f;
  K.h0 = false; K.h1 = false;
  if (K.c0 >= 0) {
    float tx0 = (a0.x - pos.x) * ix, tx1 = (b0.x - pos.x) * ix;
    float ty0 = (a0.y - pos.y) * iy, ty1 = (b0.y - pos.y) * iy;
    float tz0 = (a0.z - pos.z) * iz, tz1 = (b0.z - pos.z) * iz;
    K.tn0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    K.h0 = !(K.tn0 > tf || tf < -1e-6f) && (all || !(K.tn0 > fmaxf(w.o3, w.o7)));
  }
  if (K.c1 >= 0) {
    float tx0 = (a1.x - pos.x) * ix, tx1 = (b1.x - pos.x) * ix;
    float ty0 = (a1.y - pos.y) * iy, ty1 = (b1.y - pos.y) * iy;
    float tz0 = (a1.z - pos.z) * iz, tz1 = (b1.z - pos.z) * iz;
    K.tn1 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    K.h1 = !(K.tn1 > tf || tf < -1e-6f) && (all || !(K.tn1 > fmaxf(w.o3, w.o7)));
  }
  return K;
}

/* The walk's stack.  With ss set (a walk kernel: this thread's column of
 * a shared-memory array, entry d at ss[d * bd], bd the threads of the CTA,
 * so lanes at different depths never share a bank) its first
 * RAMP_BVH_SSTACK entries live there and the rest in w.stack; without,
 * all of it is in w.stack. */
DI void stack_push(MeshWalk& w, int* ss, int bd, int v) {
  if (ss && w.sp < RAMP_BVH_SSTACK) ss[w.sp * bd] = v;
  else w.stack[w.sp] = v;
  ++w.sp;
}
DI int stack_pop(MeshWalk& w, int* ss, int bd) {
  --w.sp;
  return (ss && w.sp < RAMP_BVH_SSTACK) ? ss[w.sp * bd] : w.stack[w.sp];
}

/* continue into the nearer hit inner child and keep the other on the stack;
 * with none, take the next node off the stack (-1 when it is empty).
 * false: the stack would overflow (the status flag is raised) */
DI bool mesh_descend(MeshWalk& w, const MeshKids& K, StatusDev* st, int* ss = nullptr,
                     int bd = 0) {
  const bool i0 = K.h0 && K.c0 == 0, i1 = K.h1 && K.c1 == 0;
  if (i0 && i1) {
    if (w.sp + 1 > RAMP_BVH_STACK) { raise_flag(st, RAMP_F_BVH_STACK); return false; }
    const bool first0 = !(K.tn1 < K.tn0);
    stack_push(w, ss, bd, first0 ? K.r1 : K.r0);
    w.node = first0 ? K.r0 : K.r1;
  } else if (i0) {
    w.node = K.r0;
  } else if (i1) {
    w.node = K.r1;
  } else {
    w.node = w.sp > 0 ? stack_pop(w, ss, bd) : -1;
  }
  return true;
}

/* one inner node of the walk: test both children, the triangles of the
 * leaf children that were hit, then move on.  Returns 1 while nodes
 * remain, 0 when the walk is over, -1 when the stack would overflow (the
 * intersection is then false and the status flag raised). */
DI int mesh_step(const CompDev& c, MeshWalk& w, StatusDev* st) {
  const MeshKids K = mesh_kids(c, w);
  /* the triangles of the leaf children that were hit, as one range */
  const int n0 = (K.h0 && K.c0 > 0) ? K.c0 : 0, n1 = (K.h1 && K.c1 > 0) ? K.c1 : 0;
  for (int j = 0; j < n0 + n1; ++j) mesh_tri(c, w, j < n0 ? K.r0 + j : K.r1 + (j - n0));
  if (!mesh_descend(w, K, st)) return -1;
  return w.node >= 0 ? 1 : 0;
}

/* one inner node without its triangles: the hit leaf children's triangles
 * become the range [tb, te), to be tested by mesh_tri.  The caller visits
 * only with an empty range and a node left.  false: stack overflow */
DI bool mesh_visit(const CompDev& c, MeshWalk& w, StatusDev* st, int* ss = nullptr, int bd = 0) {
  const MeshKids K = mesh_kids(c, w);
  const int n0 = (K.h0 && K.c0 > 0) ? K.c0 : 0, n1 = (K.h1 && K.c1 > 0) ? K.c1 : 0;
  /* sibling leaves: the second's triangles follow the first's (r1 = r0 + c0) */
  w.tb = n0 > 0 ? K.r0 : K.r1;
  w.te = n1 > 0 ? K.r1 + n1 : K.r0 + n0;
  if (n0 == 0 && n1 == 0) w.te = w.tb;
  return mesh_descend(w, K, st, ss, bd);
}

DI bool mesh_walk_over(const MeshWalk& w) { return w.tb >= w.te && w.node < 0; }

/* the records of a finished walk (mesh.cl:114-129): interior parity, then
 * the entering and exiting hits if they come before the current record */
DI bool mesh_end(const CompDev& c, Nt& n, Is& s, const MeshRec& w) {
  /* each record's point is pos + vel * t of the hit that set it (the
     values the reference stores with it; n is the ray the walk began
     with); t = 1e8 and the point 0 when there was none */
  const V3 pos = npos(n), vel = nvel(n);
  float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f, o3 = w.o3;
  float o4 = 0.0f, o5 = 0.0f, o6 = 0.0f, o7 = w.o7;
  if (o3 < 1e8f) { o0 = pos.x + vel.x * o3; o1 = pos.y + vel.y * o3; o2 = pos.z + vel.z * o3; }
  if (o7 < 1e8f) { o4 = pos.x + vel.x * o7; o5 = pos.y + vel.y * o7; o6 = pos.z + vel.z * o7; }
  if ((c.gi[0] == 1) && (w.num_intersections % 2 == 1)) {
    o4 = o0; o5 = o1; o6 = o2; o7 = o3;
  } else if ((c.gi[0] == 1) && (w.num_intersections % 2 == 0)) {
    return false;
  }
  if (o3 < s.t1) {
    s.x1 = o0; s.y1 = o1; s.z1 = o2; s.t1 = o3;
    s.x2 = o4; s.y2 = o5; s.z2 = o6; s.t2 = o7;
    if (c.scat == RAMP_S_ATTENUATE) { n.sd = w.chord > 0.0 ? (float)w.chord : 0.0f; n.wr |= WR_SD; }
    return true;
  }
  return false;
}

DI bool g_mesh(const CompDev& c, Nt& n, Is& s, StatusDev* st) {
  MeshWalk w;
  if (!mesh_begin(c, n, w)) return false;
  int k;
  while ((k = mesh_step(c, w, st)) > 0) {
  }
  if (k < 0) return false;
  return mesh_end(c, n, s, mesh_rec(w));
}

#endif /* RAMP_MESH_CUH */
