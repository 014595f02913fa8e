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
 * with a chopper, and then, where the next component is one, an on-axis
 * unrotated GCylinderExt without restore as its target.  Why the bounds
 * hold there:
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
 *  - the target (cylinder_ext.cl:3-53): the cylinder accepts a neutron
 *    only where its line crosses the cylinder's box; one it does not
 *    accept dies there (terminate.cl: no intersection, no restore).
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
 * neutron outside the assumptions (vz <= 0, within the slack of a wall at
 * the entrance of a guide whose entrance plane is wider than the guide, y
 * + R not clearly positive, angles beyond 1e4 rad) gets no claim from
 * there on.  A neutron that would instead miss a plane,
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
    if (c.geom == RAMP_G_CYL_EXT) {
      /* the run's target, after its last chopper: a cylinder of radius r
         about the y axis through (0, 0, zc), height h.  It accepts a
         neutron only where its line meets x^2 + (z - zc)^2 < r^2 with the
         exit point at |y| < h/2 (cylinder_ext.cl:3-53), so within the box
         |x| < r, |y| < h/2, |z - zc| <= r; one whose line certainly stays
         outside that box over z in [zc - r, zc + r] dies there */
      const float r = c.gp[0], hh = 0.5f * c.gp[1];
      float xlo = 1e30f, xhi = -1e30f, ylo = 1e30f, yhi = -1e30f;
      for (int e = 0; e < 2; ++e) {
        const float ze = e ? zc + r : zc - r;
        const float de = ze - z0;
        const float xe = x0 + mx * de, ye = y0 + my * de;
        const float exe = ex + (ux + 4e-6f * nb * fabsf(sx)) * fabsf(de) + 1e-6f * fabsf(xe);
        const float eye = ey + (uy + 4e-6f * nb * fabsf(sy)) * fabsf(de) + 1e-6f * fabsf(ye);
        xlo = fminf(xlo, xe - exe); xhi = fmaxf(xhi, xe + exe);
        ylo = fminf(ylo, ye - eye); yhi = fmaxf(yhi, ye + eye);
      }
      return xlo >= r || xhi <= -r || ylo >= hh || yhi <= -hh;
    }
    if (c.scat == RAMP_S_GUIDE) {
      /* a neutron that certainly misses the entrance plane dies there
         (plane.cl:3-52: |x| < width/2 and |y| < height/2 to hit it) */
      if (fabsf(xc) - exc >= 0.5f * c.gp[0] || fabsf(yc) - eyc >= 0.5f * c.gp[1]) return true;
      /* folding needs known slopes and an entry inside the walls.  With an
         entrance no wider than the guide every neutron the plane accepts
         starts inside them (|x| < width/2 <= a); one within the slack of a
         wall folds there too: the bounce loop takes the wall it flies
         towards at once, whatever the sign of that time (guide.cl:66-85),
         and the fold moves the point by less than the slack */
      const float a = 0.5f * c.sp[0], b = 0.5f * c.sp[1], l = c.sp[4];
      if (ux > 0.0f || uy > 0.0f) return false;
      if ((0.5f * c.gp[0] > a || 0.5f * c.gp[1] > b) &&
          (!(fabsf(xc) < a - exc) || !(fabsf(yc) < b - eyc)))
        return false;
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
    if (c.scat != RAMP_S_CHOPPER) continue;   /* the run's target: no speed bound */
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

/* true: no neutron with 1 / speed = iv can pass chopper q of the run */
LA_FN bool speed_chopper_blocks(const SpeedRun& R, int q, float iv) {
  const float t0 = iv * R.a0[q] - 1e-9f, t1 = iv * R.a1[q] + 1e-9f;
  const float c0 = R.fr[q] * (t0 - R.ph[q]), c1 = R.fr[q] * (t1 - R.ph[q]);
  const float dlo = fminf(c0, c1) - R.wide[q];
  const float dhi = fmaxf(c0, c1) + R.wide[q];
  if (!(fabsf(dlo) < 1e4f) || !(fabsf(dhi) < 1e4f)) return false;
  const float h = R.hb[q] + 1e-6f * fmaxf(fabsf(dlo), fabsf(dhi));
  /* no multiple of the slit period within [dlo - h, dhi + h] */
  const float klo = ceilf((dlo - h) * R.iTg[q]), khi = floorf((dhi + h) * R.iTg[q]);
  return klo > khi;
}

/* true: no neutron with 1 / speed = iv can pass every chopper of the
 * prepared run.  iv may carry a relative error of a few 1e-7 (an
 * approximate reciprocal square root): the time slack is 1e-5 of it. */
LA_FN bool speed_run_blocks(const SpeedRun& R, float iv) {
  if (!(iv > 0.0f) || !(iv < 1e30f)) return false;
  for (int q = 0; q < R.n; ++q)
    if (speed_chopper_blocks(R, q, iv)) return true;
  return false;
}

/* reorder the prepared choppers by blocked[q] (how many of a sample of
 * speeds chopper q blocks), the most first, so that the histories the run
 * retires leave the test loop early; the answer of speed_run_blocks does
 * not depend on the order */
LA_FN void speed_run_sort(SpeedRun* R, const int* blocked) {
  int key[SPEED_RUN_MAX];
  for (int q = 0; q < R->n; ++q) key[q] = blocked[q];
  for (int q = 1; q < R->n; ++q)          /* insertion sort, stable */
    for (int j = q; j > 0 && key[j] > key[j - 1]; --j) {
      const int kk = key[j]; key[j] = key[j - 1]; key[j - 1] = kk;
      float* arr[7] = {R->a0, R->a1, R->ph, R->fr, R->wide, R->hb, R->iTg};
      for (int f = 0; f < 7; ++f) {
        const float x = arr[f][j]; arr[f][j] = arr[f][j - 1]; arr[f][j - 1] = x;
      }
    }
}

/* ---- the speed table: verdicts for cells of the energy draw ------------
 * A flat or MCont moderator draws a neutron's energy first:
 * E = E_min + (E_max - E_min) u with u the reference's u01 of one Threefry
 * word x (flat_mod.cl, cont_mod.cl:36; u01fixedpt_closed_closed_32_24 reads
 * bits 6-30 of x and is non-decreasing in them), and 1 / speed is
 * 1 / (SE2V sqrt(E)).  A cell is the set of words with the same bits 19-30
 * (SPEED_CELLS cells); u, E and 1 / speed are each a chain of correctly
 * rounded operations monotone in those bits, so the 1 / speed of every word
 * of a cell lies between the values at its two ends.  speed_chopper_blocks
 * is likewise a chain of monotone operations in 1 / speed (products and
 * sums with constants, min, max, |.| of a monotone value, ceil, floor), so
 * over the cell's range every intermediate value lies between bounds taken
 * at the range's ends.  From those bounds a cell gets SPEED_BLOCKED when
 * every 1 / speed in it is blocked by one chopper, SPEED_KEPT when no
 * chopper blocks any, else SPEED_MIXED; a history in a BLOCKED or KEPT cell
 * gets from the table exactly the answer speed_run_blocks would give it,
 * and the others compute their speed and take speed_run_blocks. */
#define SPEED_CELLS 4096
#define SPEED_CELL_SHIFT 19         /* cell = bits 19-30 of the word */
#define SPEED_MIXED 0
#define SPEED_BLOCKED 1
#define SPEED_KEPT 2

struct SpeedTab {
  SpeedRun run;                   /* ordered (speed_run_sort) */
  float e0, de;                   /* E_min and E_max - E_min of the cells */
  int ncell;                      /* 0: no cells, every history takes speed_run_blocks */
  int pad;
  uint8_t cell[SPEED_CELLS];
};
#define SPEED_TAB_WORDS ((int)(sizeof(SpeedTab) / 4))

/* u01fixedpt_closed_closed_32_24 (Random123 u01fixedpt.h:137-140), as the
 * moderator's draw computes it */
LA_FN float la_u01(uint32_t i) {
  return (float)((i & 0x7fffffc0u) + (i & 0x40u)) * (1.0f / 2147483648.0f);
}

/* 1 / speed of a neutron of energy e (meV): correctly rounded square root
 * and division, both monotone */
LA_FN float speed_iv(float e) { return 1.0f / (RC_SE2V * sqrtf(e)); }

/* 1 / speed of the energy drawn from word x */
LA_FN float speed_iv_of_word(uint32_t x, float e0, float de) {
  return speed_iv(e0 + de * la_u01(x));
}

/* the 1 / speed range [*lo, *hi] of the words of cell c */
LA_FN void speed_word_cell(int c, float e0, float de, float* lo, float* hi) {
  const uint32_t first = (uint32_t)c << SPEED_CELL_SHIFT;
  const uint32_t last = first | ((1u << SPEED_CELL_SHIFT) - 1u);   /* bit 31 is not read */
  const float a = speed_iv_of_word(first, e0, de), b = speed_iv_of_word(last, e0, de);
  *lo = fminf(a, b);
  *hi = fmaxf(a, b);
}

/* SPEED_BLOCKED, SPEED_KEPT or SPEED_MIXED for chopper q over iv in [lo, hi] */
LA_FN int speed_chopper_range(const SpeedRun& R, int q, float lo, float hi) {
  float c0[2], c1[2];
  for (int e = 0; e < 2; ++e) {
    const float iv = e ? hi : lo;
    const float t0 = iv * R.a0[q] - 1e-9f, t1 = iv * R.a1[q] + 1e-9f;
    c0[e] = R.fr[q] * (t0 - R.ph[q]);
    c1[e] = R.fr[q] * (t1 - R.ph[q]);
  }
  const float c0n = fminf(c0[0], c0[1]), c0x = fmaxf(c0[0], c0[1]);
  const float c1n = fminf(c1[0], c1[1]), c1x = fmaxf(c1[0], c1[1]);
  const float dlo_n = fminf(c0n, c1n) - R.wide[q], dlo_x = fminf(c0x, c1x) - R.wide[q];
  const float dhi_n = fmaxf(c0n, c1n) + R.wide[q], dhi_x = fmaxf(c0x, c1x) + R.wide[q];
  if (!(dlo_n == dlo_n) || !(dlo_x == dlo_x) || !(dhi_n == dhi_n) || !(dhi_x == dhi_x))
    return SPEED_MIXED;
  const float mlo = fmaxf(fabsf(dlo_n), fabsf(dlo_x)), mhi = fmaxf(fabsf(dhi_n), fabsf(dhi_x));
  const float hb = R.hb[q], hx = R.hb[q] + 1e-6f * fmaxf(mlo, mhi);
  const float T = R.iTg[q];
  /* every iv of the cell blocked: the widest window holds no multiple of
     the period, and no iv of the cell falls out through the 1e4 guard */
  if (mlo < 1e4f && mhi < 1e4f && ceilf((dlo_n - hx) * T) > floorf((dhi_x + hx) * T))
    return SPEED_BLOCKED;
  /* no iv of the cell blocked: the narrowest window holds a multiple */
  if (ceilf((dlo_x - hb) * T) <= floorf((dhi_n + hb) * T)) return SPEED_KEPT;
  return SPEED_MIXED;
}

/* the verdict of a range of iv over the whole run */
LA_FN int speed_cell_verdict(const SpeedRun& R, float lo, float hi) {
  if (!(lo > 0.0f) || !(hi < 1e30f) || !(lo <= hi)) return SPEED_MIXED;
  bool all_kept = true;
  for (int q = 0; q < R.n; ++q) {
    const int v = speed_chopper_range(R, q, lo, hi);
    if (v == SPEED_BLOCKED) return SPEED_BLOCKED;
    if (v != SPEED_KEPT) all_kept = false;
  }
  return all_kept ? SPEED_KEPT : SPEED_MIXED;
}

/* cells over the energies [e0, e0 + de] (none unless both are finite) */
LA_FN void speed_tab_range(SpeedTab* T, float e0, float de) {
  T->e0 = e0;
  T->de = de;
  T->ncell = (e0 == e0 && de == de && fabsf(e0) < 1e30f && fabsf(de) < 1e30f) ? SPEED_CELLS : 0;
}

/* true: no neutron whose energy draw gave word x can pass the run (the
 * table's answer where its cell has one, else speed_run_blocks) */
LA_FN bool speed_tab_blocks(const SpeedTab& T, uint32_t x) {
  if (T.ncell > 0) {
    const int v = T.cell[(x >> SPEED_CELL_SHIFT) & (SPEED_CELLS - 1)];
    if (v == SPEED_BLOCKED) return true;
    if (v == SPEED_KEPT) return false;
  }
  return speed_run_blocks(T.run, speed_iv_of_word(x, T.e0, T.de));
}

#ifdef __CUDACC__
/* Called by every thread of a CTA of blockDim.x (a multiple of 32) threads,
 * R and blocked (SPEED_RUN_MAX ints) in shared memory: thread 0 prepares
 * the run at component 0 for a flat or MCont source with parameters p
 * (RampSource.p: p[0..4] the geometry, p[5..6] the energy range); each
 * thread then takes one energy of an even grid over the range and counts
 * the choppers that block it, and thread 0 orders the choppers by those
 * counts.  R->n = 0 when `on` is false. */
__device__ __forceinline__ void speed_run_setup(SpeedRun* R, int* blocked, bool on,
                                                const CompDev* comps, int nl, const float* p) {
  if (threadIdx.x == 0) {
    R->n = 0;
    if (on) speed_run_prepare(comps, 0, nl, p[0], p[1], p[2], p[3], p[4], R);
  }
  if (threadIdx.x < SPEED_RUN_MAX) blocked[threadIdx.x] = 0;
  __syncthreads();
  const int nq = R->n;
  if (nq > 1) {
    const float e = p[5] + (p[6] - p[5]) * (((float)threadIdx.x + 0.5f) / (float)blockDim.x);
    const float iv = speed_iv(e);
    for (int q = 0; q < nq; ++q) {
      const unsigned m = __ballot_sync(0xffffffffu, speed_chopper_blocks(*R, q, iv));
      if ((threadIdx.x & 31) == 0 && m != 0u) atomicAdd(&blocked[q], __popc(m));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && nq > 1) speed_run_sort(R, blocked);
  __syncthreads();
}

/* One CTA's share of a speed table written to dst (SPEED_TAB_WORDS words):
 * SPEED_CELLS / blockDim.x CTAs, CTA `cta` deciding cells [cta blockDim.x,
 * (cta + 1) blockDim.x) and CTA 0 also writing the run and the cell
 * layout; T and blocked in shared memory.  The run is the one at component
 * 0 (nl components) for a flat or MCont source with parameters p; the
 * cells are those of the energy draw's word over [E_min, E_max]. */
__device__ __forceinline__ void speed_tab_build(uint32_t* dst, SpeedTab* T, int* blocked,
                                                const CompDev* comps, int nl, const float* p,
                                                int cta) {
  speed_run_setup(&T->run, blocked, true, comps, nl, p);
  if (threadIdx.x == 0) speed_tab_range(T, p[5], p[6] - p[5]);
  __syncthreads();
  const int c = cta * (int)blockDim.x + (int)threadIdx.x;
  if (c < SPEED_CELLS) {
    int v = SPEED_MIXED;
    if (T->ncell > 0) {
      float lo, hi;
      speed_word_cell(c, T->e0, T->de, &lo, &hi);
      v = speed_cell_verdict(T->run, lo, hi);
    }
    reinterpret_cast<uint8_t*>(dst)[offsetof(SpeedTab, cell) + c] = (uint8_t)v;
  }
  if (cta == 0) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(T);
    for (int k = threadIdx.x; k < (int)(offsetof(SpeedTab, cell) / 4); k += blockDim.x)
      dst[k] = w[k];
  }
}

/* a speed table from dst into shared memory T, every thread of the CTA */
__device__ __forceinline__ void speed_tab_load(SpeedTab* T, const uint32_t* src) {
  uint32_t* w = reinterpret_cast<uint32_t*>(T);
  for (int k = threadIdx.x; k < SPEED_TAB_WORDS; k += blockDim.x) w[k] = src[k];
  __syncthreads();
}
#endif

#endif /* RAMP_LOOKAHEAD_H */
