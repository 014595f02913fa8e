/*
 * lookahead.h — the chopper look-ahead of split fused launches
 * (RampTune.cull).  From a neutron's state before a run of on-axis
 * components (straight guides and disk choppers) it bounds when and where
 * the neutron meets each component's plane, and tells whether some chopper
 * certainly stops it or it certainly misses a guide's entrance.  Compiled
 * for the device (the end of stage A) and for the host
 * (ramp_debug_chopper_cull, with which the bound is checked against the CPU
 * restatement of the reference kernels).
 *
 * The run (checked by chopper_run in abi.cu): components of one linear
 * block, each unrotated, centred on the z axis (x = y = 0), with a z-normal
 * GPlane and no restore, at non-decreasing z without overlaps: straight
 * SGuides (w1 = w2, h1 = h2) and SChopper components in any order, ending
 * with a chopper.  Why the bounds hold there:
 *  - time.  Nothing in the run changes vz: the frame transforms are the
 *    identity on velocities; a straight guide's wall normals have no z
 *    component (guide.cl:39-43 with w1 = w2: ww = hh = 0, so the bounce
 *    leaves vz - d * 0 = vz); planes and choppers do not touch velocities.
 *    So the time at a chopper plane is t + (zc - z) / vz, up to the
 *    rounding of the segment times and z steps the kernels add up.
 *  - transverse position.  Inside a straight guide of half-width a the
 *    motion is the unfolded line u(z) = x_e + (vx / vz)(z - z_e) reflected
 *    at x = +-a (the bounce loop, guide.cl:49-135, reflects at one wall at
 *    a time, x and y independently); after the exit the neutron flies on
 *    from its last bounce along the folded line to the next component.  A
 *    reflection changes |vx| by a few ulp (about 5e-7 relative); when the
 *    folded exit point lies within the slack of a wall, the last bounce may
 *    fall on either side of the exit plane, and both signs of vx after the
 *    exit are allowed (a later guide then ends the look-ahead).
 *  - a guide entrance (plane.cl:3-52): a neutron whose line meets the plane
 *    outside its rectangle by more than the slack misses it and dies.
 *  - a chopper (chopper.cl:4-59): the neutron passes only if the distance
 *    from freq (t - |phase|) + e - atan2(x, y + R), e in [-jitter, jitter),
 *    to the nearest multiple of 2 pi / n_slits is at most
 *    atan2(w, y + R) / 2.  atan2(x, Y) is monotone in x and in Y for Y > 0,
 *    so its range over the box of (x, y) is taken at corners, and
 *    atan2(w, Y) <= w / Y.
 * Every slack is far above the rounding it covers (time: 1e-5 relative
 * plus a micrometre of z per bounce; position: 2e-5 m plus 4e-6 of the
 * guide path per bounce so far; angle: 1e-4 rad plus 1e-6 relative, which
 * also covers the truncated atan series and products with reciprocals).  A
 * neutron outside the assumptions (vz <= 0, at a guide entrance within the
 * slack of a wall, y + R not clearly positive, angles beyond 1e4 rad) gets
 * no claim from there on.  A neutron that would instead miss a plane,
 * leave a guide at zero weight or exceed its bounce limit dies in the
 * reference as well, so with only tallies observable it may be retired
 * either way.
 */
#ifndef RAMP_LOOKAHEAD_H
#define RAMP_LOOKAHEAD_H

#include "rmath.h"
#include "plan.h"

#if defined(__CUDACC__)
#define LA_FN static __host__ __device__ __forceinline__
#else
#define LA_FN static inline
#endif

/* the folded position of the unfolded coordinate u in a guide of
 * half-width a (ia = 1/a), x = a - |((u + a) mod 4a) - 2a|; *sgn is +1
 * where the neutron moves along the unfolded line, -1 against it; *amb
 * when x lies within `slack` of a wall */
LA_FN float la_fold(float u, float a, float ia, float slack, float* sgn, bool* amb) {
  const float p = 4.0f * a;
  float m = u + a;
  m = m - p * floorf(m * (0.25f * ia));
  if (m < 0.0f) m += p;
  if (m >= p) m -= p;
  const bool up = m < 2.0f * a;
  const float x = up ? m - a : 3.0f * a - m;
  *sgn = up ? 1.0f : -1.0f;
  *amb = !(a - fabsf(x) > slack);
  return x;
}

/* atan(r): for |r| <= 1/4 the alternating series to r^7, whose error is
 * below the next term, r^9/9 < 5e-7 (the angle slack covers it), else the
 * library's atan2 */
LA_FN float la_atan(float r) {
  if (fabsf(r) <= 0.25f) {
    const float r2 = r * r;
    return r * (1.0f - r2 * (0.333333343f - r2 * (0.2f - r2 * 0.142857149f)));
  }
  return rm_atan2f(r, 1.0f);
}

/* true: the neutron at (x, y, z) with velocity (vx, vy, vz) and time t,
 * in the laboratory frame before component k, cannot pass every chopper
 * of the run comps[k .. k + nl) (or misses a guide entrance of it, which
 * kills it as well).  Divisions are replaced by products with reciprocals
 * where the slack covers their extra rounding; a chopper's aux[0] is its
 * slit period and aux[1] the reciprocal of it. */
LA_FN bool chopper_run_blocks(const CompDev* comps, int k, int nl, float x, float y, float z,
                              float vx, float vy, float vz, float t) {
  if (!(vz > 0.0f) || nl <= 0) return false;
  const float ivz = 1.0f / vz;
  const float sx = vx * ivz, sy = vy * ivz;
  /* the neutron's line: (x0, y0) at z0 with slopes (mx, my); after a guide
     exit near a wall the sign of a slope is open (mx = 0, ux = |sx|) */
  float x0 = x, y0 = y, z0 = z, mx = sx, my = sy, ux = 0.0f, uy = 0.0f;
  float ex = 2e-5f, ey = 2e-5f;   /* position slack (m) */
  float nb = 0.0f;                /* bounces so far, for the slope and time slack */
  for (int j = k; j < k + nl; ++j) {
    const CompDev& c = comps[j];
    const float zc = c.pos[2];
    const float dz = zc - z0;
    if (!(dz >= -1e-6f)) return false;
    /* where the line meets this component's plane; the slope error of
       earlier bounces carries on over dz */
    const float xc = x0 + mx * dz, yc = y0 + my * dz;
    const float exc = ex + (ux + 4e-6f * nb * fabsf(sx)) * fabsf(dz) + 1e-6f * fabsf(xc);
    const float eyc = ey + (uy + 4e-6f * nb * fabsf(sy)) * fabsf(dz) + 1e-6f * fabsf(yc);
    if (c.scat == RAMP_S_GUIDE) {
      /* a neutron that certainly misses the entrance plane dies there
         (plane.cl:3-52: |x| < width/2 and |y| < height/2 to hit it) */
      if (fabsf(xc) - exc >= 0.5f * c.gp[0] || fabsf(yc) - eyc >= 0.5f * c.gp[1]) return true;
      /* folding needs known slopes and an entry inside the walls */
      const float a = 0.5f * c.sp[0], b = 0.5f * c.sp[1], l = c.sp[4];
      if (ux > 0.0f || uy > 0.0f) return false;
      if (!(fabsf(xc) < a - exc) || !(fabsf(yc) < b - eyc)) return false;
      const float ia = 1.0f / a, ib = 1.0f / b;
      const float dux = mx * l, duy = my * l;
      const float nbx = floorf(fabsf(dux) * (0.5f * ia)) + 2.0f;
      const float nby = floorf(fabsf(duy) * (0.5f * ib)) + 2.0f;
      if (!(nbx < 1e4f) || !(nby < 1e4f)) return false;
      ex = exc + 4e-6f * (nb + nbx) * (fabsf(dux) + a);
      ey = eyc + 4e-6f * (nb + nby) * (fabsf(duy) + b);
      nb += nbx + nby;
      float gx, gy;
      bool ax, ay;
      x0 = la_fold(xc + dux, a, ia, ex, &gx, &ax);
      y0 = la_fold(yc + duy, b, ib, ey, &gy, &ay);
      z0 = zc + l;
      ux = ax ? fabsf(mx) : 0.0f;
      mx = ax ? 0.0f : gx * mx;
      uy = ay ? fabsf(my) : 0.0f;
      my = ay ? 0.0f : gy * my;
      continue;
    }
    /* a disk chopper */
    const float tc = t + (zc - z) * ivz;
    const float et = 1e-5f * fabsf(tc) + (1e-5f * fabsf(zc - z) + 1e-6f * (nb + 10.0f)) * ivz + 1e-9f;
    const float sw = c.sp[0], R = c.sp[1], freq = c.sp[2], phase = c.sp[3], jit = c.sp[4];
    const float iTg = c.aux[1];
    const float Ylo = yc - eyc + R, Yhi = yc + eyc + R;
    if (!(Ylo > 1e-3f) || !(iTg > 0.0f)) continue;
    const float iYlo = 1.0f / Ylo, iYhi = 1.0f / Yhi;
    const float xlo = xc - exc, xhi = xc + exc;
    const float th_hi = la_atan(xhi * (xhi >= 0.0f ? iYlo : iYhi));
    const float th_lo = la_atan(xlo * (xlo >= 0.0f ? iYhi : iYlo));
    const float c0 = freq * (tc - et - fabsf(phase)), c1 = freq * (tc + et - fabsf(phase));
    const float dlo = fminf(c0, c1) - fabsf(jit) - th_hi;
    const float dhi = fmaxf(c0, c1) + fabsf(jit) - th_lo;
    if (!(fabsf(dlo) < 1e4f) || !(fabsf(dhi) < 1e4f)) continue;
    const float h = 0.5f * fabsf(sw) * iYlo + 1e-4f + 1e-6f * fmaxf(fabsf(dlo), fabsf(dhi));
    /* no multiple of the slit period within [dlo - h, dhi + h] */
    const float klo = ceilf((dlo - h) * iTg), khi = floorf((dhi + h) * iTg);
    if (klo > khi) return true;
  }
  return false;
}

/* The speed look-ahead.  For a flat or MCont moderator (flat_mod.cl,
 * cont_mod.cl:11-72: emission at time 0 from a uniform point of a p0 x p1
 * rectangle at z = 0 towards a uniform point of a p2 x p3 target window at
 * distance p4) a neutron's speed v is known after its first draw, and its
 * direction lies in a cone: |vx / vz| <= (|p0| + |p2|) / (2 p4), likewise
 * y, and vz >= v / sqrt(1 + sx^2 + sy^2).  Along the run vz does not change
 * (see above), so the time at a chopper plane lies in [z / v, z / vz_min];
 * the transverse position is within the moderator rectangle widened by the
 * cone before the first guide, within a guide's walls inside it, and within
 * the walls widened by the cone after its exit.  A chopper whose slits are
 * closed over all of that stops the neutron.  Everything but v is the same
 * for every neutron of a launch: speed_run_prepare computes it once per
 * chopper, speed_run_blocks applies it to one speed. */
#define SPEED_RUN_MAX 16          /* choppers of a run the bound uses */
struct SpeedRun {
  int n;                          /* choppers prepared */
  float a0[SPEED_RUN_MAX];        /* earliest time x v (with its slack) */
  float a1[SPEED_RUN_MAX];        /* latest time x v (with its slack) */
  float ph[SPEED_RUN_MAX];        /* |phase| */
  float fr[SPEED_RUN_MAX];        /* freq */
  float wide[SPEED_RUN_MAX];      /* |jitter| + the largest |atan2(x, y + R)| */
  float hb[SPEED_RUN_MAX];        /* half the largest slit angle, plus slack */
  float iTg[SPEED_RUN_MAX];       /* 1 / slit period */
};

LA_FN void speed_run_prepare(const CompDev* comps, int k, int nl, float p0, float p1, float p2,
                             float p3, float p4, SpeedRun* R) {
  R->n = 0;
  if (!(p4 > 0.0f) || nl <= 0) return;
  const float sx = 0.5f * (fabsf(p0) + fabsf(p2)) / p4, sy = 0.5f * (fabsf(p1) + fabsf(p3)) / p4;
  const float cmin = (1.0f - 1e-5f) / sqrtf(1.0f + sx * sx + sy * sy);
  if (!(cmin > 0.0f)) return;
  const float icmin = 1.0f / cmin;
  /* |x| <= X + sx |z - z0| (and y) beyond the last guide exit z0 */
  float X = 0.5f * fabsf(p0), Y = 0.5f * fabsf(p1), z0 = 0.0f;
  float nb = 0.0f;                /* bounces the guides can take, for the time slack */
  for (int j = k; j < k + nl && R->n < SPEED_RUN_MAX; ++j) {
    const CompDev& c = comps[j];
    const float zc = c.pos[2];
    const float dz = zc - z0;
    if (!(dz >= -1e-6f)) return;
    const float Xc = X + sx * fabsf(dz), Yc = Y + sy * fabsf(dz);
    if (c.scat == RAMP_S_GUIDE) {
      const float a = 0.5f * c.sp[0], b = 0.5f * c.sp[1], l = c.sp[4];
      /* a neutron entering beside the walls (an entrance plane wider than
         the guide) is not bounded by them: the later choppers get no claim */
      if (!(0.5f * c.gp[0] <= a) || !(0.5f * c.gp[1] <= b)) return;
      nb += floorf(sx * l / (2.0f * a)) + floorf(sy * l / (2.0f * b)) + 4.0f;
      if (!(nb < 1e6f)) return;
      X = a + 2e-5f;
      Y = b + 2e-5f;
      z0 = zc + l;
      continue;
    }
    /* a disk chopper (chopper.cl:4-59): the time in [zc / v, zc / vz_min]
       widened by 1e-5 of it and a micrometre of z per bounce, the angle
       atan2(x, y + R) within +-atan(Xc / (R - Yc)) */
    const float ex = 2e-5f + 1e-6f * Xc, ey = 2e-5f + 1e-6f * Yc;
    const float sw = c.sp[0], Rr = c.sp[1];
    const float Ylo = Rr - Yc - ey;
    if (!(Ylo > 1e-3f) || !(c.aux[1] > 0.0f)) continue;
    const float e1 = (1e-5f * zc * icmin + (1e-5f * zc + 1e-6f * (nb + 10.0f)) * icmin);
    const int q = R->n++;
    R->a0[q] = zc - e1;
    R->a1[q] = zc * icmin + e1;
    R->ph[q] = fabsf(c.sp[3]);
    R->fr[q] = c.sp[2];
    R->wide[q] = fabsf(c.sp[4]) + la_atan((Xc + ex) / Ylo);
    R->hb[q] = 0.5f * fabsf(sw) / Ylo + 1e-4f;
    R->iTg[q] = c.aux[1];
  }
}

/* true: no neutron of speed v can pass every chopper of the prepared run */
LA_FN bool speed_run_blocks(const SpeedRun& R, float v) {
  if (!(v > 0.0f)) return false;
  const float iv = 1.0f / v;
  for (int q = 0; q < R.n; ++q) {
    const float t0 = iv * R.a0[q] - 1e-9f, t1 = iv * R.a1[q] + 1e-9f;
    const float c0 = R.fr[q] * (t0 - R.ph[q]), c1 = R.fr[q] * (t1 - R.ph[q]);
    const float dlo = fminf(c0, c1) - R.wide[q];
    const float dhi = fmaxf(c0, c1) + R.wide[q];
    if (!(fabsf(dlo) < 1e4f) || !(fabsf(dhi) < 1e4f)) continue;
    const float h = R.hb[q] + 1e-6f * fmaxf(fabsf(dlo), fabsf(dhi));
    /* no multiple of the slit period within [dlo - h, dhi + h] */
    const float klo = ceilf((dlo - h) * R.iTg[q]), khi = floorf((dhi + h) * R.iTg[q]);
    if (klo > khi) return true;
  }
  return false;
}

#endif /* RAMP_LOOKAHEAD_H */
