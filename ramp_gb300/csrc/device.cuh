/*
 * device.cuh — the per-neutron chain as device functions over a neutron
 * held in registers.  Shared by the plain per-component kernels
 * (plain.cu) and the fused persistent kernel (fused.cu).
 *
 * Every function restates one reference OpenCL kernel (cited) with the
 * same sequence of FP32 operations, so that with -fmad=false and the
 * shared rmath.h library the results are bit-identical to the CPU oracle.
 * Differences in structure, not in arithmetic: the frame transform uses a
 * rotation matrix precomputed on the host (the reference recomputes the
 * same nine products per work-item), a linear component's five kernels
 * (transform, intersect, terminate, scatter, untransform) run back to back
 * on registers, and the intersection record lives in registers (at the
 * start of every linear component it always holds the reset value).
 */
#ifndef RAMP_DEVICE_CUH
#define RAMP_DEVICE_CUH

#include <stdint.h>
#include "rmath.h"
#include "rconst.h"
#include "plan.h"

#define DI __device__ __forceinline__

/* ------------------------------------------------------------------ */
/* neutron record in registers (NOTES:3-14)                            */
/* ------------------------------------------------------------------ */
struct Nt {
  float x, y, z, vx, vy, vz, px, py, pz, p, t, sb, sc, sd, se, die;
  uint32_t wr;   /* lanes sc/sd/se/die written since the last store */
};
#define WR_SC 1u
#define WR_SD 2u
#define WR_SE 4u
#define WR_DIE 8u

struct Is {
  float x1, y1, z1, t1, x2, y2, z2, t2;
};

DI void is_reset(Is& s) {
  s.x1 = 0.0f; s.y1 = 0.0f; s.z1 = 0.0f; s.t1 = RC_T_RESET;
  s.x2 = 0.0f; s.y2 = 0.0f; s.z2 = 0.0f; s.t2 = RC_T_RESET;
}
DI void set_die(Nt& n, float v) { n.die = v; n.wr |= WR_DIE; }
DI void set_sc(Nt& n, uint32_t idx) { n.sc = (float)idx; n.wr |= WR_SC; }

/* ------------------------------------------------------------------ */
/* float3 helpers (OpenCL built-ins, left-to-right dot)                 */
/* ------------------------------------------------------------------ */
struct V3 { float x, y, z; };
DI V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
DI V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
DI V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
DI V3 mul(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
DI float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DI float len3(V3 a) { return sqrtf(dot(a, a)); }
DI V3 normalize(V3 a) {
  float d = dot(a, a);
  if (d == 0.0f) return a;
  float inv = 1.0f / sqrtf(d);
  return v3(a.x * inv, a.y * inv, a.z * inv);
}
DI V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
DI bool all_eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
DI V3 npos(const Nt& n) { return v3(n.x, n.y, n.z); }
DI V3 nvel(const Nt& n) { return v3(n.vx, n.vy, n.vz); }
DI V3 npol(const Nt& n) { return v3(n.px, n.py, n.pz); }
DI void set_pos(Nt& n, V3 v) { n.x = v.x; n.y = v.y; n.z = v.z; }
DI void set_vel(Nt& n, V3 v) { n.vx = v.x; n.vy = v.y; n.vz = v.z; }
DI void set_pol(Nt& n, V3 v) { n.px = v.x; n.py = v.y; n.pz = v.z; }
DI V3 ip1(const Is& s) { return v3(s.x1, s.y1, s.z1); }
DI V3 ip2(const Is& s) { return v3(s.x2, s.y2, s.z2); }

/* ------------------------------------------------------------------ */
/* Threefry-4x32-20 (Salmon et al., SC'11), written for the GPU: the key */
/* schedule is built once per neutron and the constant key and counter  */
/* words fold into immediates.  Its adds are written x * one + y, with  */
/* `one` a kernel argument equal to 1 that the compiler cannot fold, so */
/* that they issue as integer multiply-adds on the FMA pipe, beside the */
/* rotates and xors on the ALU pipe; mod 2^32 the value is x + y.        */
/* ------------------------------------------------------------------ */
DI uint32_t rotl(uint32_t x, int r) { return __funnelshift_l(x, x, r); }

#define TF_E(a, b) x0 = x1 * one + x0; x1 = rotl(x1, a) ^ x0; \
                   x2 = x3 * one + x2; x3 = rotl(x3, b) ^ x2;
#define TF_O(a, b) x0 = x3 * one + x0; x3 = rotl(x3, a) ^ x0; \
                   x2 = x1 * one + x2; x1 = rotl(x1, b) ^ x2;
#define TF_INJ(s, k0, k1, k2, k3) x0 = (k0) * one + x0; x1 = (k1) * one + x1; \
                                  x2 = (k2) * one + x2; x3 = ((k3) + (s)) * one + x3;

DI void tf20(uint32_t& x0, uint32_t& x1, uint32_t& x2, uint32_t& x3, uint32_t K0, uint32_t K1,
             uint32_t K2, uint32_t K3, uint32_t K4, uint32_t one) {
  x0 = K0 * one + x0; x1 = K1 * one + x1; x2 = K2 * one + x2; x3 = K3 * one + x3;
  TF_E(10, 26) TF_O(11, 21) TF_E(13, 27) TF_O(23, 5) TF_INJ(1u, K1, K2, K3, K4)
  TF_E(6, 20) TF_O(17, 11) TF_E(25, 10) TF_O(18, 20) TF_INJ(2u, K2, K3, K4, K0)
  TF_E(10, 26) TF_O(11, 21) TF_E(13, 27) TF_O(23, 5) TF_INJ(3u, K3, K4, K0, K1)
  TF_E(6, 20) TF_O(17, 11) TF_E(25, 10) TF_O(18, 20) TF_INJ(4u, K4, K0, K1, K2)
  TF_E(10, 26) TF_O(11, 21) TF_E(13, 27) TF_O(23, 5) TF_INJ(5u, K0, K1, K2, K3)
}

#define TF_C1 0xf00dcafeu
#define TF_C2 0xdeadbeefu
#define TF_C3 0xbeeff00du
#define TF_K1 0xdecafbadu
#define TF_K2 0xfacebeadu
#define TF_K3 0x12345678u
#define TF_PARITY 0x1BD11BDAu

/* word x of threefry4x32({c0,C1,C2,C3}, {tid,K1,K2,K3}) (rand.h:7-16) */
DI uint32_t tf_ref_x(uint32_t c0, uint32_t tid, uint32_t k4, uint32_t one) {
  uint32_t x0 = c0, x1 = TF_C1, x2 = TF_C2, x3 = TF_C3;
  tf20(x0, x1, x2, x3, tid, TF_K1, TF_K2, TF_K3, k4, one);
  return x0;
}

/* u01fixedpt_closed_closed_32_24 (Random123 u01fixedpt.h:137-140) */
DI float u01cc(uint32_t i) {
  return (float)((i & 0x7fffffc0u) + (i & 0x40u)) * (1.0f / 2147483648.0f);
}

struct Rng {
  uint32_t tid, k1, k2, k4;   /* key words 0..2 and the parity word */
  uint32_t one;               /* 1 (tf20) */
  int mode;
  uint32_t blk;               /* native mode: cached block index       */
  uint32_t w0, w1, w2, w3;
};

DI void rng_init(Rng& r, int mode, uint32_t tid, uint32_t variant, uint32_t run_seed,
                 uint32_t one) {
  r.mode = mode;
  r.tid = tid;
  r.one = one;
  if (mode == 0) {
    r.k1 = TF_K1; r.k2 = TF_K2;
  } else {
    r.k1 = variant; r.k2 = run_seed;
  }
  r.k4 = TF_PARITY ^ tid ^ r.k1 ^ r.k2 ^ TF_K3;
  r.blk = 0xffffffffu;
  r.w0 = r.w1 = r.w2 = r.w3 = 0u;
}

/* rand() — mcramp/include/rand.h:4-21: counter word 0 is (uint)sb, sb is
 * advanced by one.  Native mode reads word (sb & 3) of block sb >> 2.
 * draw_word gives the Threefry word, draw the number rand() returns. */
DI uint32_t draw_word(Nt& n, Rng& r) {
  uint32_t c = (uint32_t)n.sb;
  uint32_t x;
  if (r.mode == 0) {
    x = tf_ref_x(c, r.tid, r.k4, r.one);
  } else {
    uint32_t b = c >> 2;
    if (b != r.blk) {
      uint32_t x0 = b, x1 = TF_C1, x2 = TF_C2, x3 = TF_C3;
      tf20(x0, x1, x2, x3, r.tid, r.k1, r.k2, TF_K3, r.k4, r.one);
      r.w0 = x0; r.w1 = x1; r.w2 = x2; r.w3 = x3;
      r.blk = b;
    }
    uint32_t j = c & 3u;
    x = (j == 0) ? r.w0 : (j == 1) ? r.w1 : (j == 2) ? r.w2 : r.w3;
  }
  n.sb += 1.0f;
  return x;
}
DI float draw(Nt& n, Rng& r) { return u01cc(draw_word(n, r)); }

/* ------------------------------------------------------------------ */
/* status                                                               */
/* ------------------------------------------------------------------ */
DI void raise_flag(StatusDev* st, unsigned int f) { atomicOr(&st->flags, f); }

/* tally add with warp aggregation of lanes hitting the same bin of the
 * same histogram (lanes of one warp can reach this code for different
 * components of the same kind, so the histogram address is part of the
 * match key) */
/* Float atomic addition on the GPU (red/atom.add.f32) flushes subnormal
 * operands to zero; terms are flushed here before any aggregation so that
 * a tally is the FTZ sum of its terms whatever the grouping (the oracle
 * flushes the same way). */
DI float ftz(float x) { return fabsf(x) < 1.17549435e-38f ? copysignf(0.0f, x) : x; }

/* shared memory of a whole-chain launch with private tallies */
extern __shared__ float ramp_dyn_smem[];

/* A detector's histograms: its CTA-private copies in shared memory when the
 * launch privatises them (merged into global memory as the CTA ends), else
 * the global ones. */
DI void tally_add(const CompDev& c, long long idx, float p) {
  float* h = c.tally;
  float* he = c.tally_err;
  if (c.priv_off >= 0) {
    h = ramp_dyn_smem + c.priv_off;
    he = c.tally_err ? h + c.tally_len : nullptr;
  }
  unsigned m = __activemask();
  unsigned peers = __match_any_sync(m, idx) & __match_any_sync(m, (unsigned long long)h);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  p = ftz(p);
  float s = p, s2 = ftz(p * p);
  if (__popc(peers) > 1) {
    float a = 0.0f, a2 = 0.0f;
    unsigned rest = peers;
    while (rest) {
      int src = __ffs(rest) - 1;
      rest &= rest - 1;
      float q = __shfl_sync(peers, p, src);
      a += q;
      a2 += ftz(q * q);
    }
    s = a; s2 = a2;
  }
  if (lane == leader) {
    atomicAdd(h + idx, s);
    if (he) atomicAdd(he + idx, s2);
  }
}

/* ------------------------------------------------------------------ */
/* adjoint context: the chain functions take a context type D; NoDiff    */
/* compiles every derivative hook away (the forward kernels), AdjDiff    */
/* accumulates d log p / d theta per neutron and, at the loss detector,  */
/* adds dL/dH_bin * p * d log p / d theta to the gradient.               */
/* ------------------------------------------------------------------ */
struct NoDiff {
  static constexpr bool on = false;
  static constexpr bool pol = true;   /* the spin lanes are output */
  static constexpr bool rec = false;  /* record the loss detector's neutrons */
  static constexpr bool tally = true; /* add to the tallies */
};

/* Whole-chain kernels output tallies only, and no component turns the spin
 * into a weight, a position or a branch: the spin lanes are dead there.
 * Their draws are still taken (the RNG counter must advance as it does
 * with them), their trigonometry and rotations are skipped. */
struct TallyOnly : NoDiff {
  static constexpr bool pol = false;
};

/* First pass of the adjoint: trace without tallies and record the index
 * of every neutron the loss detector counts (once per neutron); only those
 * neutrons carry a gradient term, and only they are replayed with AdjDiff. */
template <bool TALLY>
struct RecorderT {
  static constexpr bool on = false;
  static constexpr bool pol = false;
  static constexpr bool rec = true;
  static constexpr bool tally = TALLY;    /* also the forward histogram */
  uint32_t idx;                     /* this neutron's index in the launch */
  bool done;
  uint32_t* list;
  unsigned long long* count;
  int64_t cap;
  DI void hit() {
    if (done) return;
    done = true;
    const unsigned long long k = atomicAdd(count, 1ull);
    if ((int64_t)k < cap) list[k] = idx;
  }
};
using Recorder = RecorderT<false>;

struct AdjDiff {
  static constexpr bool on = true;
  static constexpr bool pol = false;
  static constexpr bool rec = false;
  static constexpr bool tally = false;
  float dlog[RAMP_MAX_DIFF];
  double* grad;      /* nslot accumulators, global                       */
  int nslot;
  int lr;            /* add likelihood-ratio terms of branch choices     */
  DI void reset(int n, double* g, int lr_) {
    nslot = n; grad = g; lr = lr_;
    for (int k = 0; k < RAMP_MAX_DIFF; ++k) dlog[k] = 0.0f;
  }
  DI void add(int slot, float v) { if (slot >= 0) dlog[slot] += v; }
  /* the neutron is tallied by the loss detector with weight p in a bin of
   * adjoint g */
  DI void tallied(float g, float p) {
    float w = g * p;
    if (w == 0.0f) return;
    for (int k = 0; k < nslot; ++k) atomicAdd(grad + k, (double)w * (double)dlog[k]);
  }
};

/* ------------------------------------------------------------------ */
/* moderators                                                           */
/* ------------------------------------------------------------------ */
/* maxwell_energy_distn — cont_mod.cl:4-9 (pow(x,1.5) as x*sqrt(x)) */
DI float maxwell(float E, float T) {
  float rootE = sqrtf(E);
  float overKT = 1.0f / (RC_K_B * T);
  return 2.0f * rootE / sqrtf(RC_PI) * (overKT * sqrtf(overKT)) * rm_expf(-E * overKT);
}
/* the same with 1/(k_B T) and its 3/2 power from the plan */
DI float maxwell_pre(float E, float overKT, float okc) {
  float rootE = sqrtf(E);
  return 2.0f * rootE / sqrtf(RC_PI) * okc * rm_expf(-E * overKT);
}

/* MISIS table read: entries outside the table read as 0 (the reference
 * reads past both ends for a deviate below the first flux value or above
 * the last, isis_mod.cl:27-38) */
DI float isis_at(const float* __restrict__ t, int64_t len, int64_t i) {
  return (i >= 0 && i < len) ? __ldg(t + i) : 0.0f;
}

/* find_closest_in_cdf (isis_mod.cl:4-13): the index before the first entry
 * above val, 0 when none is; by bisection (the table is non-decreasing and
 * val >= 0, so entries past its end, read as 0, never qualify) */
DI int isis_cdf(const float* __restrict__ t, int len, float val) {
  int lo = 0, hi = len;               /* first index with t[i] - val > 0 */
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((__ldg(t + mid) - val) > 0.0f) hi = mid;
    else lo = mid + 1;
  }
  return lo < len ? lo - 1 : 0;
}

/* energy and time of an MISIS history (isis_mod.cl:31-70); returns the
 * energy in meV, the emission time in t0 */
DI float isis_sample(const SrcDev& s, Nt& n, Rng& r, float& t0) {
  const float* __restrict__ flux = s.tab[0];
  const float* __restrict__ tb = s.tab[1];
  const float* __restrict__ eb = s.tab[2];
  const float* __restrict__ ei = s.tab[3];
  const int nt = s.n_t, ne = s.n_e;
  const int64_t nflux = (int64_t)(ne - 1) * nt;
  float deviate = s.p[14] * draw(n, r);
  const int idx = isis_cdf(flux, (int)nflux, deviate);
  const int Epnt = isis_cdf(ei, ne, deviate);
  int Tpnt = (int)fmodf((float)idx, (float)nt);
  if (Tpnt >= nt - 1) Tpnt -= 1;
  float time_val = isis_at(tb, nt, Tpnt);
  const float time_range = isis_at(tb, nt, Tpnt + 1) - isis_at(tb, nt, Tpnt);
  const int64_t row = (int64_t)Epnt * nt;
  const float time_spread = isis_at(flux, nflux, row + Tpnt + 1) - isis_at(flux, nflux, row + Tpnt);
  float R = deviate - isis_at(flux, nflux, row + Tpnt);
  R /= time_spread;
  time_val += time_range * R;
  const float ener_spread = isis_at(ei, ne, Epnt + 1) - isis_at(ei, ne, Epnt);
  const int i0 = (Epnt > 3) ? Epnt - 3 : 0;
  const int i1 = ((ne - Epnt - 1) > 3) ? Epnt + 3 : (ne - 1);
  deviate = isis_at(ei, ne, Epnt) + ener_spread * draw(n, r);
  float acc = 0.0f;                     /* Lagrange interpolation of the edge */
  for (int i = i0; i <= i1; i++) {
    float Pj = 1.0f;
    const float ei_i = isis_at(ei, ne, i);
    for (int j = i0; j <= i1; j++)
      if (j != i) Pj *= (deviate - isis_at(ei, ne, j)) / (ei_i - isis_at(ei, ne, j));
    Pj *= isis_at(eb, ne, i);
    acc += Pj;
  }
  t0 = time_val;
  return acc;
}

/* MCont weight sum_i I_i M(E; T_i) / M(k_B T_i; T_i) / N (cont_mod.cl:22-31) */
template <class D>
DI float cont_weight(const SrcDev& s, float E_val, int32_t num_sim, D* dx) {
  float E_J = RC_EV_J * E_val;
  float M = s.p[8] * maxwell_pre(E_J, s.okt[0], s.okc[0]) / s.dmax[0];
  if (!(s.zero_terms & 2u)) M += s.p[10] * maxwell_pre(E_J, s.okt[1], s.okc[1]) / s.dmax[1];
  if (!(s.zero_terms & 4u)) M += s.p[12] * maxwell_pre(E_J, s.okt[2], s.okc[2]) / s.dmax[2];
  if constexpr (D::on) {
    /* weight I M(E;T)/M(kT;T) = I sqrt(x) e^(1-x), x = E/kT, for the
       common temperature T of the three terms: d log/dT = (x - 1/2)/T */
    if (s.dslot_T >= 0 && M != 0.0f) {
      float acc = 0.0f;
      for (int q = 0; q < 3; ++q) {
        const float T = s.p[7 + 2 * q], I = s.p[8 + 2 * q];
        const float term = I * maxwell(E_J, T) / s.dmax[q];
        const float x = E_J / (RC_K_B * T);
        acc += term * (x - 0.5f) / T;
      }
      dx->add(s.dslot_T, acc / M);
    }
  }
  return M / (float)num_sim;
}

/* the weight of a flat or MCont history of energy E_val (flat_mod.cl:26,
 * cont_mod.cl:39-47) */
template <class D = NoDiff>
DI float source_weight(const SrcDev& s, float E_val, int32_t num_sim, D* dx = nullptr) {
  return (s.kind == RAMP_SRC_CONT) ? cont_weight<D>(s, E_val, num_sim, dx)
                                   : 1.0f / (float)num_sim;
}

/* generate_neutrons — flat_mod.cl:4-50, cont_mod.cl:11-72, isis_mod.cl:15-104.
 * EXT = false compiles the kernel without the extended kinds (the MISIS
 * source here, the TAS components in scatter): a smaller whole-chain
 * kernel for chains that do not use them.  WEIGHT = false (flat and MCont
 * sources only) leaves the energy in n.p for source_weight to turn into the
 * weight later, with the same operations: a kernel that may retire the
 * history first skips the weight for those it retires. */
template <class D = NoDiff, bool EXT = true, bool WEIGHT = true>
DI void generate(const SrcDev& s, Nt& n, float old_sb, int32_t num_sim, int32_t seed, Rng& r,
                 D* dx = nullptr) {
  n.x = n.y = n.z = n.vx = n.vy = n.vz = n.px = n.py = n.pz = 0.0f;
  n.p = n.t = n.sc = n.sd = n.se = n.die = 0.0f;
  n.wr = 0;
  n.sb = (float)seed + old_sb;
  float E_val, t0 = 0.0f;
  if (EXT && s.kind == RAMP_SRC_ISIS) {
    E_val = isis_sample(s, n, r, t0);
    n.p = s.p[13] * s.p[14] * 6.2415093e+12f / (float)num_sim;
  } else {
    const float E_min = s.p[5], E_max = s.p[6];
    float E_range = (E_max - E_min);
    E_val = E_min + E_range * draw(n, r);
    n.p = WEIGHT ? source_weight<D>(s, E_val, num_sim, dx) : E_val;
  }
  n.x = s.p[0] * (0.5f - draw(n, r));
  n.y = s.p[1] * (0.5f - draw(n, r));
  n.z = 0.0f;
  float vel = RC_SE2V * sqrtf(E_val);
  float Dx = s.p[2] * (0.5f - draw(n, r)) - n.x;
  float Dy = s.p[3] * (0.5f - draw(n, r)) - n.y;
  set_vel(n, mul(vel, normalize(v3(Dx, Dy, s.p[4]))));
  if constexpr (D::pol) {
    float theta = 2 * RC_PI * draw(n, r);
    float phi = rm_acosf(1 - 2 * draw(n, r));
    float sp, cp, st, ct;
    rm_sincosf(phi, &sp, &cp);
    rm_sincosf(theta, &st, &ct);
    n.px = sp * ct;
    n.py = sp * st;
    n.pz = cp;
  } else {
    /* the spin's two draws only advance the counter: their values are
       unused, and a native-mode block is recomputed from its index */
    n.sb += 1.0f;
    n.sb += 1.0f;
  }
  n.t = t0;
  n.die = 0.0f;
}

/* ------------------------------------------------------------------ */
/* frame transform — frametransform.cl:4-42, geom.h:21-87               */
/* pos/vel are always rotated (an identity matrix gives the same values */
/* as the reference's explicit products), the spin only when the       */
/* component is rotated.                                                 */
/* ------------------------------------------------------------------ */
DI V3 rot_fwd(const float* R, V3 v) {
  return v3(dot(v3(R[0], R[1], R[2]), v), dot(v3(R[3], R[4], R[5]), v),
            dot(v3(R[6], R[7], R[8]), v));
}
DI V3 rot_inv(const float* R, V3 v) {
  return v3(dot(v3(R[0], R[3], R[6]), v), dot(v3(R[1], R[4], R[7]), v),
            dot(v3(R[2], R[5], R[8]), v));
}
template <bool POL = true>
DI void transform(const CompDev& c, Nt& n) {
  set_pos(n, sub(npos(n), v3(c.pos[0], c.pos[1], c.pos[2])));
  set_pos(n, rot_inv(c.R, npos(n)));
  set_vel(n, rot_inv(c.R, nvel(n)));
  if (POL && c.rotated) set_pol(n, rot_inv(c.R, npol(n)));
}
template <bool POL = true>
DI void untransform(const CompDev& c, Nt& n) {
  set_pos(n, rot_fwd(c.R, npos(n)));
  set_pos(n, add(npos(n), v3(c.pos[0], c.pos[1], c.pos[2])));
  set_vel(n, rot_fwd(c.R, nvel(n)));
  if (POL && c.rotated) set_pol(n, rot_fwd(c.R, npol(n)));
}

/* rotate_about_axis — geom.h:1-19 */
DI V3 rotate_about_axis(float angle, V3 a, V3 v) {
  float s, c;
  rm_sincosf(angle, &s, &c);
  float Rxx = c + a.x * a.x * (1 - c);
  float Rxy = a.x * a.y * (1 - c) - a.z * s;
  float Rxz = a.x * a.z * (1 - c) + a.y * s;
  float Ryx = a.y * a.x * (1 - c) + a.z * s;
  float Ryy = c + a.y * a.y * (1 - c);
  float Ryz = a.y * a.z * (1 - c) - a.x * s;
  float Rzx = a.z * a.x * (1 - c) - a.y * s;
  float Rzy = a.z * a.y * (1 - c) + a.x * s;
  float Rzz = c + a.z * a.z * (1 - c);
  return v3(Rxx * v.x + Rxy * v.y + Rxz * v.z, Ryx * v.x + Ryy * v.y + Ryz * v.z,
            Rzx * v.x + Rzy * v.y + Rzz * v.z);
}

/* reflectivity_func — include/ref.h:3-53 (beta = 0 unless set) */
DI float reflectivity(float q, float R0, float Qc, float alpha, float m, float W) {
  float beta = 0.0f, arg;
  if (W == 0.0f && alpha == 0.0f) {
    m = m * 0.9853f + 0.1978f;
    W = -0.0002f * m + 0.0022f;
    alpha = 0.2304f * m + 5.0944f;
    beta = -7.6251f * m + 68.1137f;
    if (m <= 3) { alpha = m; beta = 0; }
  }
  arg = W > 0 ? (q - m * Qc) / W : 11;
  if (arg > 10 || m <= 0 || Qc <= 0 || R0 <= 0) return 0.0f;
  if (m < 1) { Qc *= m; m = 1; }
  if (q <= Qc) return R0;
  return R0 * 0.5f * (1 - rm_tanhf(arg)) * (1 - alpha * (q - Qc) + beta * (q - Qc) * (q - Qc));
}

/* ------------------------------------------------------------------ */
/* geometry kernels: return true when they store iidx = comp_idx        */
/* ------------------------------------------------------------------ */
/* plane.cl:3-52 */
DI bool g_plane(const CompDev& c, const Nt& n, Is& s) {
  const float width = c.gp[0], height = c.gp[1];
  V3 vel = nvel(n), pos = npos(n);
  float t = 0.0f, x = 0.0f, y = 0.0f;
  if (c.gi[0] == 0) {
    t = (-pos.z) / vel.z; x = pos.x + t * vel.x; y = pos.y + t * vel.y;
  } else if (c.gi[0] == 1) {
    t = (-pos.x) / vel.x; x = pos.z + t * vel.z; y = pos.y + t * vel.y;
  }
  if ((fabsf(x) < width / 2.0f) && (fabsf(y) < height / 2.0f) && t < s.t1 && t < s.t2 &&
      t > 0.0f && dot(vel, v3(0.0f, 0.0f, 1.0f)) > 0.f) {
    V3 h = add(pos, mul(t, vel));
    s.x1 = h.x; s.y1 = h.y; s.z1 = h.z;
    s.x2 = h.x; s.y2 = h.y; s.z2 = h.z;
    s.t1 = t; s.t2 = t;
    return true;
  }
  return false;
}

/* cylinder_ext.cl:3-53 and banana.cl:3-55 */
template <bool BANANA>
DI bool g_cyl(const CompDev& c, const Nt& n, Is& s) {
  const float radius = c.gp[0], height = c.gp[1];
  float ppx = n.x, ppz = n.z, pvx = n.vx, pvz = n.vz;
  float a = pvx * pvx + pvz * pvz;
  float b = 2.0f * (ppx * pvx + ppz * pvz);
  float cc = (ppx * ppx + ppz * ppz) - radius * radius;
  float quotient = b * b - 4.0f * a * cc;
  float sq = sqrtf(quotient);
  float t1 = (-b - sq) / (2.f * a);
  float t2 = (-b + sq) / (2.f * a);
  float yt2 = n.y + t2 * n.vy;
  bool window = true;
  if (BANANA) {
    /* (mintheta < theta2) < maxtheta, banana.cl:38 */
    const float mintheta = c.gp[2], maxtheta = c.gp[3];
    if (maxtheta > 1.0f) {
      window = true;
    } else if (!(maxtheta > 0.0f)) {
      window = false;
    } else {
      float hx = ppx + t2 * pvx, hz = ppz + t2 * pvz;
      float d2 = hx * hx + hz * hz;
      float nz = hz;
      if (d2 != 0.0f) { float inv = 1.0f / sqrtf(d2); nz = hz * inv; hx = hx * inv; }
      float theta2 = rm_acosf(hx * 0.0f + nz * 1.0f);
      window = (float)(mintheta < theta2) < maxtheta;
    }
  }
  if ((quotient > 0.0f) && ((-height / 2.0f) < yt2) && (yt2 < (height / 2)) && window) {
    bool ok = BANANA ? (t2 < s.t1 && t1 < 0.0f && t2 > 0.0f)
                     : (t1 < s.t1 && t1 > 0.0f && t2 > 0.0f);
    if (ok) {
      V3 p1 = add(npos(n), mul(t1, nvel(n)));
      V3 p2 = add(npos(n), mul(t2, nvel(n)));
      s.x1 = p1.x; s.y1 = p1.y; s.z1 = p1.z; s.t1 = t1;
      s.x2 = p2.x; s.y2 = p2.y; s.z2 = p2.z; s.t2 = t2;
      return true;
    }
  }
  return false;
}

/* sphere.cl:3-42 and sphere_int.cl:3-41 */
template <bool INTERIOR>
DI bool g_sphere(const CompDev& c, const Nt& n, Is& s) {
  V3 pos = npos(n), vel = nvel(n);
  float r = c.gp[0];
  float a = dot(vel, vel);
  float b = 2.0f * (dot(vel, pos));
  float cc = dot(pos, pos) - r * r;
  float quotient = b * b - 4.0f * a * cc;
  if (quotient > 0.0f) {
    float sq = sqrtf(quotient);
    float d1 = (-b - sq) / (2.f * a);
    float d2 = (-b + sq) / (2.f * a);
    if (!INTERIOR) {
      if (d1 < s.t1 && d1 > 0.f) {
        V3 p1 = add(pos, mul(d1, vel)), p2 = add(pos, mul(d2, vel));
        s.x1 = p1.x; s.y1 = p1.y; s.z1 = p1.z; s.t1 = d1;
        s.x2 = p2.x; s.y2 = p2.y; s.z2 = p2.z; s.t2 = d2;
        return true;
      }
    } else {
      if (d1 < 0.0f && d2 < s.t1) {
        V3 p2 = add(pos, mul(d2, vel));
        s.x1 = p2.x; s.y1 = p2.y; s.z1 = p2.z; s.t1 = d2;
        s.x2 = p2.x; s.y2 = p2.y; s.z2 = p2.z; s.t2 = d2;
        return true;
      }
    }
  }
  return false;
}

/* box.cl:3-53 */
DI bool g_box(const CompDev& c, const Nt& n, Is& s) {
  V3 pos = npos(n), vel = nvel(n);
  V3 A = v3(-c.gp[0] / 2.0f, -c.gp[1] / 2.0f, -c.gp[2] / 2.0f);
  V3 B = v3(c.gp[0] / 2.0f, c.gp[1] / 2.0f, c.gp[2] / 2.0f);
  V3 dA = sub(A, pos), dB = sub(B, pos);
  float t1 = dA.x / vel.x, t2 = dB.x / vel.x, t3 = dA.y / vel.y;
  float t4 = dB.y / vel.y, t5 = dA.z / vel.z, t6 = dB.z / vel.z;
  float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
  float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
  /* box.cl:10,52: on a miss the kernel stores its never-initialised local
     record, a store of an undefined value that the OpenCL compiler drops:
     the record keeps what earlier components left */
  if (tmax < 0.0f) return false;
  if (tmin > tmax) return false;
  V3 p1 = add(pos, mul(tmin, vel)), p2 = add(pos, mul(tmax, vel));
  s.x1 = p1.x; s.y1 = p1.y; s.z1 = p1.z; s.t1 = tmin;
  s.x2 = p2.x; s.y2 = p2.y; s.z2 = p2.z; s.t2 = tmax;
  return true;
}

/* arm.cl:3-21 */
DI bool g_arm(Is& s) {
  s.x2 = 1.0f; s.y2 = 1.0f; s.z2 = 1.0f;
  return true;
}

#include "mesh.cuh"

/* dispatch; a mesh paired with SAttenuate leaves its chord sum in sd.
 * MESH = false compiles the kernel without the mesh hierarchy walk (its
 * 64-entry stack and live state raise register pressure in the whole
 * kernel); a plan holding a GMesh never runs such a kernel. */
template <bool MESH = true>
DI bool intersect(const CompDev& c, Nt& n, Is& s, StatusDev* st) {
  switch (c.geom) {
    case RAMP_G_PLANE: return g_plane(c, n, s);
    case RAMP_G_CYL_EXT: return g_cyl<false>(c, n, s);
    case RAMP_G_BANANA: return g_cyl<true>(c, n, s);
    case RAMP_G_SPHERE: return g_sphere<false>(c, n, s);
    case RAMP_G_SPHERE_INT: return g_sphere<true>(c, n, s);
    case RAMP_G_BOX: return g_box(c, n, s);
    case RAMP_G_ARM: return g_arm(s);
    case RAMP_G_MESH:
      if constexpr (MESH) return g_mesh(c, n, s, st);
      return false;
    default: return false;
  }
}

/* ------------------------------------------------------------------ */
/* scattering kernels                                                   */
/* ------------------------------------------------------------------ */
DI void s_finish(const CompDev& c, Nt& n, Is& s, uint32_t& ii) {
  ii = 0;
  set_sc(n, c.idx);
  is_reset(s);
}

/* reflectivity_func (ref.h:3-53) with the per-guide constants of
 * guide_aux: the same operations on the same values as reflectivity() */
DI float reflectivity_pre(float q, const float* aux, float R0) {
  const float W = aux[9];
  float arg = W > 0 ? (q - aux[12]) / W : 11;
  if (arg > 10 || aux[15] != 0.0f) return 0.0f;
  const float Qc = aux[13];
  if (q <= Qc) return R0;
  return aux[14] * (1 - rm_tanhf(arg)) * (1 - aux[10] * (q - Qc) + aux[11] * (q - Qc) * (q - Qc));
}

/* d log R / d (R0, Qc, alpha, m, W) for a bounce with momentum q, R > 0
 * (analytic derivative of reflectivity_func, ref.h:3-53) */
template <class D>
DI void guide_dlogR(const CompDev& c, float q, float R, D* dx) {
  const float R0 = c.sp[5], Qc = c.sp[6], m0 = c.sp[8];
  const float m = c.aux[8], W = c.aux[9], alpha = c.aux[10], beta = c.aux[11];
  const float Qc2 = c.aux[13];
  const bool param = (c.sp[9] == 0.0f && c.sp[7] == 0.0f);   /* m-parametrisation */
  float dR[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (q <= Qc2) {
    dR[0] = 1.0f;
  } else {
    const float arg = (q - c.aux[12]) / W;
    const float th = rm_tanhf(arg);
    const float T = 1.0f - th, dT = -(1.0f - th * th);
    const float u = q - Qc2;
    const float P = 1.0f - alpha * u + beta * u * u;
    const float R0h = 0.5f * R0;
    const float dPdQc2 = alpha - 2.0f * beta * u;
    const float dQc2dQc = (m < 1.0f) ? m : 1.0f;
    const float dQc2dm = (m < 1.0f) ? Qc : 0.0f;
    const float dargdQc = -m / W, dargdm = -Qc / W, dargdW = -arg / W;
    dR[0] = 0.5f * T * P;
    dR[1] = R0h * (dT * dargdQc * P + T * dPdQc2 * dQc2dQc);
    /* m and W, alpha, beta as the reflectivity sees them */
    float dRdm = R0h * (dT * dargdm * P + T * dPdQc2 * dQc2dm);
    float dRdW = R0h * dT * dargdW * P;
    float dRdalpha = R0h * T * (-u);
    float dRdbeta = R0h * T * u * u;
    if (!param) {
      dR[2] = dRdalpha;
      dR[3] = dRdm;
      dR[4] = dRdW;
    } else {
      /* m_eff = 0.9853 m + 0.1978; W, alpha, beta follow m_eff */
      float dalpha_dm = (m <= 3.0f) ? 1.0f : 0.2304f;
      float dbeta_dm = (m <= 3.0f) ? 0.0f : -7.6251f;
      float total = dRdm + dRdW * (-0.0002f) + dRdalpha * dalpha_dm + dRdbeta * dbeta_dm;
      dR[3] = total * 0.9853f;
      (void)m0;
    }
  }
  for (int k = 0; k < 5; ++k) dx->add(c.dslot[k], dR[k] / R);
}

/* One pass of the bounce loop of guide.cl:49-135 (the loop body with its
 * condition): i is the loop variable (reset to 0 and set to the wall hit,
 * then incremented, each pass, as in the reference), guard the hard cap.
 * Returns 1 after a bounce (loop again), 0 when the loop is over (exit
 * plane reached, cap reached or i >= max_bounces; s_guide_end follows) and
 * -1 when the neutron was retired at zero weight (nothing follows). */
template <class D = NoDiff>
DI int guide_pass(const CompDev& c, Nt& n, uint32_t& i, int& guard, StatusDev* st, D* dx,
                  const bool zx) {
  const float l = c.sp[4], R0 = c.sp[5];
  const uint32_t max_bounces = (uint32_t)c.si[0];
  const float ww = c.aux[0], hh = c.aux[1], Av = c.aux[2], Ah = c.aux[3];
  if (!(i < max_bounces)) return 0;
  if (++guard > RC_GUIDE_HARD_CAP) {
    set_die(n, 1.0f);
    raise_flag(st, RAMP_F_GUIDE_CAP);
    return 0;
  }
  float av = l * n.vx, bv = ww * n.vz, ah = l * n.vy, bh = hh * n.vz;
  float vdotn_v1 = bv + av, vdotn_v2 = bv - av, vdotn_h1 = bh + ah, vdotn_h2 = bh - ah;
  float cv1 = Av - n.z * ww, cv2 = n.x * l;
  float ch1 = Ah - n.z * hh, ch2 = n.y * l;
  float t1 = (l - n.z) / n.vz;
  i = 0;
  /* The four wall tests of guide.cl:66-85 in their order.  Of each pair of
     opposite walls one approaches the neutron (both only in a narrowing
     guide): its division is selected first and done by every lane, so a
     warp whose neutrons fly left and right divides once, not twice. */
  const bool v1 = vdotn_v1 < 0.0f, v2 = vdotn_v2 < 0.0f;
  if (v1 || v2) {
    const float tv = (v1 ? (cv1 - cv2) : (cv1 + cv2)) / (v1 ? vdotn_v1 : vdotn_v2);
    if (tv < t1) { t1 = tv; i = v1 ? 1u : 2u; }
    if (v1 && v2) {
      const float tw = (cv1 + cv2) / vdotn_v2;
      if (tw < t1) { t1 = tw; i = 2; }
    }
  }
  const bool h1 = vdotn_h1 < 0.0f, h2 = vdotn_h2 < 0.0f;
  if (h1 || h2) {
    const float th = (h1 ? (ch1 - ch2) : (ch1 + ch2)) / (h1 ? vdotn_h1 : vdotn_h2);
    if (th < t1) { t1 = th; i = h1 ? 3u : 4u; }
    if (h1 && h2) {
      const float tw = (ch1 + ch2) / vdotn_h2;
      if (tw < t1) { t1 = tw; i = 4; }
    }
  }
  if (i == 0) return 0;
  n.x = n.x + t1 * n.vx; n.y = n.y + t1 * n.vy; n.z = n.z + t1 * n.vz;
  n.t += t1;
  const bool vert = (i <= 2);
  const float wv = vert ? ww : hh;
  const float nlen2 = vert ? c.aux[4] : c.aux[6];
  const float snlen = vert ? c.aux[5] : c.aux[7];
  const float vdn = (i == 1) ? vdotn_v1 : (i == 2) ? vdotn_v2 : (i == 3) ? vdotn_h1 : vdotn_h2;
  const float q = RC_V2K * (-2.0f) * vdn / snlen;
  const float d = 2.0f * vdn / nlen2;
  if (i == 1) n.vx = n.vx - d * l;
  else if (i == 2) n.vx = n.vx + d * l;
  else if (i == 3) n.vy = n.vy - d * l;
  else n.vy = n.vy + d * l;
  n.vz = n.vz - d * wv;
  float refl = reflectivity_pre(q, c.aux, R0);
  n.p *= refl;
  if (refl < 1e-12f || refl > 1.0f) n.p = 0.0f;
  if (zx && n.p == 0.0f) {   /* retire: it can only add zeros from here */
    set_die(n, 1.0f);
    return -1;
  }
  if constexpr (D::on) {
    if (n.p != 0.0f) guide_dlogR(c, q, refl, dx);
  }
  i++;
  return 1;
}

/* guide.cl:36-37: move to the entrance plane */
DI void s_guide_begin(Nt& n, const Is& s) {
  set_pos(n, ip2(s));
  n.t += s.t2;
}

/* after the bounce loop (guide.cl:137-148) */
DI void s_guide_end(const CompDev& c, Nt& n, Is& s, uint32_t& ii, uint32_t i) {
  if (i >= (uint32_t)c.si[0]) set_die(n, 1.0f);
  s_finish(c, n, s, ii);
}

/* guide.cl:9-149 */
template <class D = NoDiff>
DI void s_guide(const CompDev& c, Nt& n, Is& s, uint32_t& ii, StatusDev* st, D* dx = nullptr,
                const bool zx = false) {
  s_guide_begin(n, s);
  uint32_t i = 0;
  int guard = 0;
  int k;
  while ((k = guide_pass<D>(c, n, i, guard, st, dx, zx)) > 0) {
  }
  if (k < 0) return;
  s_guide_end(c, n, s, ii, i);
}

/* chopper.cl:4-59 */
DI void s_chopper(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r) {
  const float slit_width = c.sp[0], radius = c.sp[1], freq = c.sp[2], phase = c.sp[3];
  const float jitter = c.sp[4];
  set_pos(n, ip2(s));
  n.t += s.t2;
  const float Tg = c.aux[0];              /* 2 pi / n_slits (si[0]), from the plan */
  float pha_error = jitter * 2.0f * (draw(n, r) - 0.5f);
  float thi_chop = freq * (n.t - fabsf(phase)) + pha_error;
  float thi_neut = rm_atan2f(n.x, n.y + radius);
  float thi_diff = fabsf(thi_chop - thi_neut);
  float ang_diff = fmodf(thi_diff, Tg);
  if (fabsf(ang_diff - Tg) < ang_diff) ang_diff = fabsf(ang_diff - Tg);
  float width = rm_atan2f(slit_width, n.y + radius);
  if (ang_diff > width / 2.0f) set_die(n, 1.0f);
  s_finish(c, n, s, ii);
}

/* sample_distn — isotropic.cl:5-73 */
DI void sample_distn(Nt& n, Rng& r, const float* __restrict__ q, const float* __restrict__ w,
                     const float* __restrict__ pw_cdf, const float* __restrict__ pq_cdf,
                     uint32_t qsamples, uint32_t wsamples, float& omega, float& Q) {
  float u = draw(n, r);
  float v = draw(n, r);
  float mindiff = 1.f;
  uint32_t w_index = 0;
  omega = 0.0f; Q = 0.0f;
  for (uint32_t i = 0; i < wsamples; i++) {
    float pc = __ldg(pw_cdf + i);
    if (pc == 1.f) break;
    if (fabsf(pc - v) < mindiff) {
      mindiff = fabsf(pc - v);
      float lo = (i > 0 ? __ldg(w + i - 1) : 0.0f);
      omega = lo + (draw(n, r)) * (__ldg(w + i) - lo);
      w_index = i;
    }
  }
  mindiff = 1.f;
  const float* row = pq_cdf + (size_t)w_index * qsamples;
  for (uint32_t i = 0; i < qsamples; i++) {
    float pc = __ldg(row + i);
    if (pc == 1.f) break;
    if (fabsf(pc - u) < mindiff) {
      mindiff = fabsf(pc - u);
      float lo = (i > 0 ? __ldg(q + i - 1) : 0.0f);
      Q = lo + (draw(n, r)) * (__ldg(q + i) - lo);
    }
  }
}

/* isotropic.cl:75-322 */
template <bool POL = true>
DI void s_isotropic(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r) {
  const float temperature = c.sp[0];
  const uint32_t transmit = (uint32_t)c.si[0];
  V3 path;
  if (all_eq(ip1(s), ip2(s))) path = sub(ip2(s), npos(n));
  else path = sub(ip2(s), ip1(s));
  float ki = RC_V2K * len3(nvel(n));
  V3 normvel = normalize(nvel(n));
  float ss0 = c.sp[3], ss1 = c.sp[6], ss2 = c.sp[9];
  float sigma_s = (ss0 + ss1 + ss2) / (2.f * ki * ki);
  float sigma_a = (c.sp[2] + c.sp[5] + c.sp[8]) * 2200.f / len3(nvel(n));
  float sigma_tot = sigma_a + sigma_s;
  float mu = (c.sp[1] + c.sp[4] + c.sp[7]) * sigma_tot * 100.f;
  float p_trans = rm_expf(-mu * len3(path));
  if (draw(n, r) < p_trans) {
    n.p *= p_trans;
    set_pos(n, add(ip2(s), mul(0.0001f, normalize(path))));
    n.t += s.t2;
    if (transmit == 0) set_die(n, 1.0f);
    s_finish(c, n, s, ii);
    return;
  }
  n.p *= (1 - p_trans) * sigma_s / sigma_tot;
  float eta = draw(n, r);
  float path_length = (-1.f / mu) * rm_logf(1 - eta * (1 - rm_expf(-mu * len3(path))));
  float u = draw(n, r);
  u *= sigma_s;
  uint32_t flag = 0;
  float b1 = ss0 / (2.f * ki * ki), b2 = (ss0 + ss1) / (2.f * ki * ki);
  if (u < b1) flag = 1;
  else if (u > b1 && u < b2) flag = 2;
  else if (u > b2) flag = 3;
  float omega = 0.0f, Q = 0.0f;
  if (flag >= 1) {
    int ch = (int)flag - 1;
    sample_distn(n, r, c.tab[4 * ch], c.tab[4 * ch + 1], c.tab[4 * ch + 2], c.tab[4 * ch + 3],
                 (uint32_t)c.si[1 + 2 * ch], (uint32_t)c.si[2 + 2 * ch], omega, Q);
  }
  if (ki * ki < (RC_E2KS * omega)) {
    set_die(n, 1.0f);
    ii = 0;
    is_reset(s);
    return;
  }
  float kf;
  if (draw(n, r) > 0.5f * rm_expf(-omega / (RC_KB * temperature))) {
    kf = sqrtf(ki * ki - RC_E2KS * omega);
    n.se = omega;
  } else {
    kf = sqrtf(ki * ki + RC_E2KS * omega);
    n.se = -omega;
  }
  n.wr |= WR_SE;
  float arg = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
  if (fabsf(arg) > 1) {
    set_die(n, 1.0f);
    ii = 0;
    is_reset(s);
    return;
  }
  float theta = rm_acosf(arg);
  V3 oldvel = nvel(n);
  float zz = -(n.vx + n.vy) / (n.vz);
  V3 perp = normalize(v3(1.f, 1.f, zz));
  float alpha = 2 * RC_PI * draw(n, r);
  perp = rotate_about_axis(alpha, normvel, perp);
  normvel = rotate_about_axis(theta, perp, normvel);
  float TOFs = path_length / len3(nvel(n));
  n.sd = Q;
  n.wr |= WR_SD;
  if (all_eq(ip1(s), ip2(s))) {
    set_pos(n, mul(path_length, path));
    n.t += TOFs;
  } else {
    set_pos(n, add(ip1(s), mul(path_length, path)));
    n.t += s.t1 + TOFs;
  }
  set_vel(n, v3(normvel.x * kf * RC_K2V, normvel.y * kf * RC_K2V, normvel.z * kf * RC_K2V));
  V3 dv = sub(oldvel, nvel(n));
  V3 q_norm = normalize(v3(dv.x * RC_V2K, dv.y * RC_V2K, dv.z * RC_V2K));
  if (!POL) {
  } else if (flag == 2) {
    const float k = -1.0f / 3.0f;
    set_pol(n, v3(n.px * k, n.py * k, n.pz * k));
  } else if (flag == 3) {
    float dp = dot(npol(n), q_norm);
    set_pol(n, v3(-q_norm.x * dp, -q_norm.y * dp, -q_norm.z * dp));
  }
  s_finish(c, n, s, ii);
}

/* powderN.cl:5-156 */
template <class D = NoDiff>
DI void s_powdern(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r, StatusDev* st,
                  D* dx = nullptr) {
  const float* __restrict__ ssv2 = c.tab[0];
  const float* __restrict__ qv = c.tab[1];
  const float sigma_abs_v = c.sp[0], d_phi = c.sp[1];
  const uint32_t num_lines = (uint32_t)c.si[0];
  const uint32_t transmit = (uint32_t)c.si[1];
  V3 path;
  if (all_eq(ip1(s), ip2(s))) path = sub(ip2(s), npos(n));
  else path = sub(ip2(s), ip1(s));
  float full_path_length = len3(path);
  float vel = len3(nvel(n));
  float sigma_abs = sigma_abs_v * 2200.0f / vel;
  float vv = vel * vel * RC_V2K * RC_V2K;
  float sum_sigma_scat = 0.0f;
  for (uint32_t j = 0; j < num_lines; j++) sum_sigma_scat += __ldg(ssv2 + j) / vv;
  float p_inter = 1 - rm_expf(-(sum_sigma_scat + sigma_abs) * full_path_length);
  /* d Sigma / d (sigma_abs * v), the descriptor value sp[0] */
  const float dSig = 2200.0f / vel;
  if (draw(n, r) > p_inter) {
    n.p *= 1 - p_inter;
    if constexpr (D::on) {
      /* weight factor exp(-Sigma L); the branch has the same probability */
      float g = -full_path_length * dSig;
      dx->add(c.dslot[0], dx->lr ? 2.0f * g : g);
    }
    set_pos(n, add(ip2(s), mul(0.0001f, normalize(path))));
    n.t += s.t2;
    if (transmit == 0) set_die(n, 1.0f);
    s_finish(c, n, s, ii);
    return;
  }
  uint32_t attempts = 0;
  float arg = 0.0f, q_chosen = 0.0f;
  while (true) {
    float u = draw(n, r);
    float v = 0.0f;
    uint32_t j = 0;
    while (v < u && j < num_lines) {
      q_chosen = __ldg(qv + j);
      v += (__ldg(ssv2 + j) / vv) / sum_sigma_scat;
      j++;
    }
    arg = q_chosen * RC_K2V / (2.0f * vel);
    if (arg < 1.0f) break;
    bool give_up = (arg > 1.0f && attempts > 2 * num_lines);
    if (give_up || attempts > RC_POWDER_HARD_CAP) {
      if (!give_up) raise_flag(st, RAMP_F_POWDER_CAP);
      set_die(n, 1.0f);
      ii = 0;
      is_reset(s);
      return;
    }
    attempts++;
  }
  float twotheta = 2.0f * rm_asinf(arg);
  const float u_depth = draw(n, r);
  float pen_depth = -rm_logf(1.0f - u_depth * (1.0f - p_inter)) / (sigma_abs + sum_sigma_scat);
  V3 beam_para = normalize(nvel(n));
  V3 beam_perp = cross(beam_para, v3(0.0f, 1.0f, 0.0f));
  if (len3(beam_perp) < 1e-3f) beam_perp = normalize(cross(beam_para, v3(1.0f, 0.0f, 0.0f)));
  else beam_perp = normalize(beam_perp);
  float phi;
  if (d_phi != 0.0f) {
    phi = (2.0f * draw(n, r) - 1.0f) * (d_phi * RC_PI / 180.0f);
    if (draw(n, r) > 0.5f) phi += RC_PI;
    phi += RC_PI / 2.0f;
  } else {
    phi = 2.0f * RC_PI * draw(n, r);
  }
  beam_perp = rotate_about_axis(phi, beam_para, beam_perp);
  beam_para = rotate_about_axis(twotheta, beam_perp, beam_para);
  if (all_eq(ip1(s), ip2(s))) {
    set_pos(n, add(npos(n), mul(pen_depth, path)));
    n.t += len3(mul(pen_depth, path)) / len3(nvel(n));
  } else {
    set_pos(n, add(ip1(s), mul(pen_depth, path)));
    n.t += s.t2 - s.t1;
  }
  set_vel(n, mul(vel, normalize(beam_para)));
  n.p *= (1 - rm_expf(-(sum_sigma_scat + sigma_abs) * pen_depth)) * sum_sigma_scat /
         (sum_sigma_scat + sigma_abs);
  if constexpr (D::on) {
    /* weight factor (1 - e^(-Sigma d)) Ss / Sigma with the depth d
       reparameterised through its inverse CDF at fixed u:
       d = -log(A)/Sigma, A = 1 - u (1 - e^(-Sigma L)) */
    const float Sig = sum_sigma_scat + sigma_abs, L = full_path_length;
    const float eL = rm_expf(-Sig * L), ed = rm_expf(-Sig * pen_depth);
    const float A = 1.0f - u_depth * (1.0f - eL);
    const float dd = u_depth * L * eL / (A * Sig) - pen_depth / Sig;
    float g = (ed * (pen_depth + Sig * dd)) / (1.0f - ed) - 1.0f / Sig;
    if (dx->lr) g += L * eL / (1.0f - eL);       /* scatter branch, probability 1 - e^(-Sigma L) */
    dx->add(c.dslot[0], g * dSig);
  }
  s_finish(c, n, s, ii);
}

/* randnorm — monochromator.cl:10-20 (Box-Muller, cosine branch) */
DI float randnorm(Nt& n, Rng& r) {
  float u1 = draw(n, r);
  float u2 = draw(n, r);
  return sqrtf(-2.0f * rm_logf(u1)) * rm_cosf(2.0f * RC_PI * u2);
}

/* GAUSS(x, 0, rms) — monochromator.cl:5-8 */
DI float gauss0(float x, float rms) {
  float d = x - 0.0f;
  return rm_expf(-d * d / (2.0f * rms * rms)) / (sqrtf(2.0f * RC_PI) * rms);
}

/* frame matrix of a rotation given by angles, as geom.h:21-53 builds it */
DI void frame_matrix(float x_a, float y_a, float z_a, float* R) {
  float sx, cx, sy, cy, sz, cz;
  rm_sincosf(x_a, &sx, &cx);
  rm_sincosf(y_a, &sy, &cy);
  rm_sincosf(z_a, &sz, &cz);
  R[0] = cy * cz;
  R[1] = -cx * sz + sx * sy * cz;
  R[2] = sx * sz + cx * sy * cz;
  R[3] = cy * sz;
  R[4] = cx * cz + sx * sy * sz;
  R[5] = -sx * cz + cx * sy * sz;
  R[6] = -sy;
  R[7] = sx * cy;
  R[8] = cx * cy;
}

/* SMonochromator — monochromator.cl:22-195: a mosaic crystal of
 * n_horizontal x n_vertical slabs (optionally curved), Bragg reflection of
 * the allowed order from the local yz plane with an anisotropic Gaussian
 * mosaic; the outgoing direction is sampled around the Bragg cone and
 * weighted by the mosaic over a 15-point Gauss-Legendre normalisation.
 * sp: slab_width, slab_height, gap, mosaic_h, mosaic_v (arc min), r0,
 * d_spacing, radius_vertical, radius_horizontal; si: n_horizontal,
 * n_vertical; tab[0], tab[1]: Gauss-Legendre nodes and weights */
DI void s_mono(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r) {
  const float slab_width = c.sp[0], slab_height = c.sp[1], gap = c.sp[2];
  const float mosaic_h = c.sp[3], mosaic_v = c.sp[4], r0 = c.sp[5], d_spacing = c.sp[6];
  const float radius_vertical = c.sp[7], radius_horizontal = c.sp[8];
  const uint32_t n_h = (uint32_t)c.si[0], n_v = (uint32_t)c.si[1];
  const float* __restrict__ gx = c.tab[0];
  const float* __restrict__ gw = c.tab[1];
  const uint32_t glen = (uint32_t)c.tab_len[0];
  set_pos(n, ip2(s));
  n.t += s.t2;
  float mos_rms_y = RC_MIN2RAD * mosaic_h / sqrtf(8.0f * rm_logf(2.0f));
  float mos_rms_z = RC_MIN2RAD * mosaic_v / sqrtf(8.0f * rm_logf(2.0f));
  float mos_rms_max = mos_rms_y > mos_rms_z ? mos_rms_y : mos_rms_z;
  float Q = 2.0f * RC_PI / d_spacing;
  float zmax = (((float)n_h * (slab_width + gap)) - gap) / 2.0f;
  float zmin = -zmax;
  float ymax = (((float)n_v * (slab_height + gap)) - gap) / 2.0f;
  float ymin = -ymax;
  if (n.z > zmin && n.z < zmax && n.y > ymin && n.y < ymax) {
    float col = ceilf((n.z - zmin) / (slab_width + gap));
    float row = ceilf((n.y - ymin) / (slab_height + gap));
    float tilt_h = radius_horizontal > 0.0f
        ? rm_asinf((col - (float)(n_h + 1) / 2.0f) * (slab_width + gap) / radius_horizontal)
        : 0.0f;
    float tilt_v = radius_vertical > 0.0f
        ? -rm_asinf((row - (float)(n_v + 1) / 2.0f) * (slab_height + gap) / radius_vertical)
        : 0.0f;
    float center_z = zmin + (col - 0.5f) * (slab_width + gap) - gap / 2.0f;
    float center_y = ymin + (row - 0.5f) * (slab_height + gap) - gap / 2.0f;
    V3 slab_pos = v3(0.0f, center_y, center_z);
    float R[9];
    frame_matrix(0.0f, tilt_h, tilt_v, R);
    set_vel(n, rot_inv(R, nvel(n)));
    set_pos(n, sub(npos(n), slab_pos));
    set_pos(n, rot_inv(R, npos(n)));
    if (fabsf(n.z) <= slab_width / 2.0f && fabsf(n.y) <= slab_height / 2.0f) {
      V3 ki = mul(RC_V2K, nvel(n));
      float ratio = -2.0f * ki.x / Q;
      float Q_order = floorf(ratio + 0.5f);
      if (Q_order == 0.0f) Q_order = ratio < 0.0f ? -1.0f : 1.0f;
      if (Q_order < 0.0f) Q_order = -Q_order;
      V3 ku = normalize(ki);
      if (Q_order > 2.0f * len3(ki) / Q) Q_order -= 1.0f;
      float q0 = Q_order * Q;
      float q0x = ratio < 0.0f ? -q0 : q0;
      float theta = rm_asinf(q0 / (2.0f * len3(ki)));
      float delta = rm_asinf(fabsf(ku.x)) - theta;
      float l12 = sqrtf(ki.y * ki.y + ki.z * ki.z);
      float p_reflect = fabsf(r0) *
          rm_expf(-ki.z * ki.z / (l12 * l12) * delta * delta / (2.0f * mos_rms_y * mos_rms_y)) *
          rm_expf(-ki.y * ki.y / (l12 * l12) * delta * delta / (2.0f * mos_rms_z * mos_rms_z));
      if (draw(n, r) <= p_reflect) {
        float cos_2theta = rm_cosf(2.0f * theta);
        float k_sin_2theta = len3(ki) * rm_sinf(2.0f * theta);
        V3 b = normalize(cross(ki, v3(q0x, 0.0f, 0.0f)));
        b = mul(k_sin_2theta, b);
        V3 a = cross(b, ku);
        float total = 0.0f;
        float mos_sample = mos_rms_max / rm_cosf(theta);
        V3 c1 = mul(cos_2theta - 1.0f, ki);
        float w = 0.0f;
        V3 q;
        for (uint32_t it = 0; it < 100; it++) {
          w = 5.0f * mos_sample;
          float sin_phi, cos_phi;
          rm_sincosf(w, &sin_phi, &cos_phi);
          q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
          q.y = q.y / mos_rms_z;
          q.z = q.z / mos_rms_y;
          if (q.z * q.z + q.y * q.y < (25.0f / (2.0f / 3.0f)) * (q.x * q.x)) break;
          mos_sample *= (2.0f / 3.0f);
        }
        for (uint32_t g = 0; g < glen; g++) {
          float phi = w * __ldg(gx + g);
          float sin_phi, cos_phi;
          rm_sincosf(phi, &sin_phi, &cos_phi);
          q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
          p_reflect = gauss0(q.z / q.x, mos_rms_y) * gauss0(q.y / q.x, mos_rms_z);
          total += __ldg(gw + g) * p_reflect;
        }
        total *= w;
        float phi = mos_sample * randnorm(n, r);
        float sin_phi, cos_phi;
        rm_sincosf(phi, &sin_phi, &cos_phi);
        q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
        p_reflect = gauss0(q.z / q.x, mos_rms_y) * gauss0(q.y / q.x, mos_rms_z);
        set_vel(n, mul(RC_K2V, add(ki, q)));
        p_reflect /= total * gauss0(phi, mos_sample);
        if (p_reflect > 1.0f) p_reflect = 1.0f;
        n.p *= p_reflect;
      }
    }
    set_pos(n, rot_fwd(R, npos(n)));
    set_pos(n, add(npos(n), slab_pos));
    set_vel(n, rot_fwd(R, nvel(n)));
  }
  s_finish(c, n, s, ii);
}

/* SPowder1 — powder1.cl:5-100: one Bragg line; the neutron scatters onto
 * the Debye-Scherrer cone at a depth drawn from the attenuation, with
 * optional phi focusing.  sp: sigma_scat*v^2, sigma_abs*v, q, d_phi */
DI void s_powder1(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r) {
  const float sigma_scat_v2 = c.sp[0], sigma_abs_v = c.sp[1], q = c.sp[2], d_phi = c.sp[3];
  n.t += s.t1;
  V3 path = sub(ip2(s), ip1(s));
  float full_path_length = len3(path);
  float vel = len3(nvel(n));
  float sigma_scat = sigma_scat_v2 / (vel * vel * RC_V2K * RC_V2K);
  float sigma_abs = sigma_abs_v * 2200.0f / vel;
  float p_scat = sigma_scat / (sigma_abs + sigma_scat);
  float p_inter = 1 - rm_expf(-(sigma_scat + sigma_abs) * full_path_length);
  float arg = q * RC_K2V / (2.0f * vel);
  if (arg > 1.0f) {
    s_finish(c, n, s, ii);
    return;
  }
  float twotheta = 2.0f * rm_asinf(arg);
  n.p *= p_scat;
  float pen_depth = -rm_logf(1.0f - draw(n, r) * (1.0f - p_inter)) / (sigma_abs + sigma_scat);
  V3 beam_para = normalize(nvel(n));
  V3 beam_perp = cross(beam_para, v3(0.0f, 1.0f, 0.0f));
  if (len3(beam_perp) < 1e-3f) beam_perp = normalize(cross(beam_para, v3(1.0f, 0.0f, 0.0f)));
  else beam_perp = normalize(beam_perp);
  float phi;
  if (d_phi != 0.0f) {
    phi = (2.0f * draw(n, r) - 1.0f) * (d_phi * RC_PI / 180.0f);
    if (draw(n, r) > 0.5f) phi += RC_PI;
    phi += RC_PI / 2.0f;
  } else {
    phi = 2.0f * RC_PI * draw(n, r);
  }
  beam_perp = rotate_about_axis(phi, beam_para, beam_perp);
  beam_para = rotate_about_axis(twotheta, beam_perp, beam_para);
  set_pos(n, add(ip1(s), mul(pen_depth, path)));
  set_vel(n, mul(vel, normalize(beam_para)));
  n.t += s.t2 - s.t1;
  n.p *= full_path_length * sigma_scat * rm_expf(-(sigma_scat + sigma_abs) * full_path_length);
  s_finish(c, n, s, ii);
}

/* SRescal — rescal.cl:5-76: picks a scattering point along the chord,
 * sends the neutron into a cone of half-angle atan(focus_r / |target|)
 * around target with final energy E0 +- dE, and records the event
 * (ki - kf, weight, energy transfer) in ev[8] (ev[3..5] are 0).
 * sp: target.x, target.y, target.z, E0, dE, focus_r */
DI void s_rescal(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r, float* ev) {
  const V3 target = v3(c.sp[0], c.sp[1], c.sp[2]);
  const float E0 = c.sp[3], dE = c.sp[4], focus_r = c.sp[5];
  V3 path = sub(ip2(s), ip1(s));
  set_pos(n, add(ip1(s), mul(draw(n, r), path)));
  V3 ki = mul(RC_V2K, nvel(n));
  float l2 = len3(target) * len3(target);
  float costhetamax = sqrtf(l2 / (focus_r * focus_r + l2));
  float theta = rm_acosf(1.0f - draw(n, r) * (1.0f - costhetamax));
  float phi = draw(n, r) * 2.0f * RC_PI;
  V3 target_perp = (target.x == 0.0f && target.z == 0.0f) ? v3(1.0f, 0.0f, 0.0f)
                                                           : v3(-target.z, 0.0f, target.x);
  V3 target_perp_perp = cross(target, target_perp);
  V3 target_final = rotate_about_axis(theta, target_perp_perp, target);
  target_final = rotate_about_axis(phi, target, target_final);
  target_final = normalize(target_final);
  float Ef = E0 + dE * (1.0f - 2.0f * draw(n, r));
  float vf = RC_SE2V * sqrtf(Ef);
  set_vel(n, mul(vf, target_final));
  V3 kf = mul(RC_V2K, nvel(n));
  float lk = len3(mul(RC_K2V, ki));
  ev[0] = ki.x - kf.x; ev[1] = ki.y - kf.y; ev[2] = ki.z - kf.z;
  ev[3] = 0.0f; ev[4] = 0.0f; ev[5] = 0.0f;
  ev[6] = n.p;
  ev[7] = RC_VS2E * (lk * lk) - Ef;
  s_finish(c, n, s, ii);
}

/* detector1D.cl:20-77 */
template <class D = NoDiff>
DI void s_det1d(const CompDev& c, Nt& n, Is& s, uint32_t& ii, StatusDev* st, D* dx = nullptr) {
  const float min_var = c.sp[0], step_var = c.sp[1], max_var = c.sp[2];
  const uint32_t var = (uint32_t)c.si[0], restore = (uint32_t)c.si[1];
  float var_val = 0.0f;
  if (var == 0) { float L = len3(nvel(n)); var_val = RC_VS2E * (L * L); }
  else if (var == 1) var_val = rm_degrees(rm_atan2f(s.x2, s.z2));
  else if (var == 2) var_val = (1.0e6f) * (n.t + s.t2);
  else if (var == 3) var_val = 2 * RC_PI / (RC_V2K * len3(nvel(n)));
  if (min_var <= var_val && var_val <= max_var) {
    uint32_t idx = (uint32_t)floorf((var_val - min_var) / step_var);
    if ((long long)idx < c.tally_len) {
      if constexpr (D::on) {
        if (c.adj_det) dx->tallied(__ldg(c.dLdH + idx), ftz(n.p));
      } else {
        if constexpr (D::rec) {
          if (c.adj_det) dx->hit();
        }
        if constexpr (D::tally) tally_add(c, idx, n.p);
      }
    } else if constexpr (D::tally) {
      if (n.p != 0.0f) atomicAdd(&st->oob, 1ull);   /* a nonzero weight was lost */
    }
  }
  if (restore == 0) {
    set_pos(n, ip2(s));
    n.t += s.t2;
    set_die(n, 1.f);
  }
  s_finish(c, n, s, ii);
}

/* axis variables, detector2D.cl:48-145 */
DI float det2d_val(uint32_t var, int axis, const Nt& n, const Is& s) {
  float X2 = s.x2, Y2 = s.y2, Z2 = s.z2;
  switch (var) {
    case 0: return X2;
    case 1: return Y2;
    case 2: return rm_degrees(rm_atan2f(X2, Z2));
    case 3: return rm_degrees(rm_atan2f(Y2, sqrtf(X2 * X2 + Z2 * Z2)));
    case 4: return rm_sign(Y2) * rm_degrees(rm_acosf(X2 / sqrtf(X2 * X2 + Y2 * Y2)));
    case 5: return (1.0e6f) * (n.t + s.t2);
    case 6: return rm_degrees(rm_atan2f(n.vx, axis == 1 ? Y2 : n.vz));
    case 7: return rm_degrees(rm_atan2f(n.vy, axis == 1 ? Y2 : n.vz));
    case 8: return 2 * RC_PI / (RC_V2K * len3(nvel(n)));
    case 9: { float L = len3(nvel(n)); return RC_VS2E * (L * L); }
    case 10: return rm_sign(X2) * rm_degrees(rm_atan2f(sqrtf(X2 * X2 + Y2 * Y2), Z2));
    default: return 0.0f;
  }
}

DI int find_idx(float val, float b0, float b1, float b2) {
  if (b0 <= val && val <= b2) return (int)roundf((val - b0) / b1);
  return -1;
}

/* detector2D.cl:31-186 */
template <class D = NoDiff>
DI void s_det2d(const CompDev& c, Nt& n, Is& s, uint32_t& ii, StatusDev* st, D* dx = nullptr) {
  int a1 = find_idx(det2d_val((uint32_t)c.si[0], 1, n, s), c.sp[0], c.sp[1], c.sp[2]);
  int a2 = find_idx(det2d_val((uint32_t)c.si[1], 2, n, s), c.sp[3], c.sp[4], c.sp[5]);
  if (!((a1 == -1) || (a2 == -1))) {
    long long flat = (long long)a1 * c.si[3] + a2;
    if (flat >= 0 && flat < c.tally_len) {
      if constexpr (D::on) {
        if (c.adj_det) dx->tallied(__ldg(c.dLdH + flat), ftz(n.p));
      } else {
        if constexpr (D::rec) {
          if (c.adj_det) dx->hit();
        }
        if constexpr (D::tally) tally_add(c, flat, n.p);
      }
    } else if constexpr (D::tally) {
      if (n.p != 0.0f) atomicAdd(&st->oob, 1ull);   /* a nonzero weight was lost */
    }
  }
  if (c.si[4] == 0) {
    set_pos(n, ip2(s));
    n.t += s.t2;
    set_die(n, 1.f);
  }
  s_finish(c, n, s, ii);
}

/* SAttenuate: weight exp(-mu L) over the mesh chord sum held in sd */
DI void s_attenuate(const CompDev& c, Nt& n, Is& s, uint32_t& ii) {
  float chord_len = n.sd * len3(nvel(n));
  n.p *= rm_expf(-c.sp[0] * chord_len);
  set_pos(n, ip2(s));
  n.t += s.t2;
  s_finish(c, n, s, ii);
}

template <class D = NoDiff, bool EXT = true, bool MESH = true>
DI void scatter(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r, StatusDev* st,
                D* dx = nullptr, const bool zx = false) {
  switch (c.scat) {
    case RAMP_S_ARM: ii = c.idx; is_reset(s); break;
    case RAMP_S_GUIDE: s_guide<D>(c, n, s, ii, st, dx, zx); break;
    case RAMP_S_CHOPPER: s_chopper(c, n, s, ii, r); break;
    case RAMP_S_ISOTROPIC: s_isotropic<D::pol>(c, n, s, ii, r); break;
    case RAMP_S_POWDERN: s_powdern<D>(c, n, s, ii, r, st, dx); break;
    case RAMP_S_DET1D: s_det1d<D>(c, n, s, ii, st, dx); break;
    case RAMP_S_DET2D: s_det2d<D>(c, n, s, ii, st, dx); break;
    case RAMP_S_COUNTER:
      if (D::tally && c.tally) atomicAdd(c.tally, n.p);
      n.se = 1.0f; n.wr |= WR_SE;
      s_finish(c, n, s, ii);
      break;
    case RAMP_S_BEAMSTOP: set_die(n, 1.0f); s_finish(c, n, s, ii); break;
    case RAMP_S_ATTENUATE: if constexpr (MESH) s_attenuate(c, n, s, ii); break;
    case RAMP_S_MONO: if constexpr (EXT) s_mono(c, n, s, ii, r); break;
    case RAMP_S_POWDER1: if constexpr (EXT) s_powder1(c, n, s, ii, r); break;
    default: break;
  }
}

/* ------------------------------------------------------------------ */
/* one component of a linear block (mcramp.py:124-157): transform,      */
/* intersect, terminate, scatter, untransform on a live neutron.  The   */
/* intersection starts at its reset value.                               */
/* ------------------------------------------------------------------ */
template <class D = NoDiff, bool EXT = true, bool MESH = true>
DI void comp_linear(const CompDev& c, Nt& n, uint32_t& ii, Rng& r, StatusDev* st,
                    D* dx = nullptr, const bool zx = false) {
  transform<D::pol>(c, n);
  Is s;
  is_reset(s);
  if (intersect<MESH>(c, n, s, st)) ii = c.idx;
  /* terminate.cl:16-18 */
  if (len3(ip2(s)) == 0.0f && c.restore == 0) set_die(n, 1.f);
  if (ii == c.idx && !(n.die > 0.f)) scatter<D, EXT, MESH>(c, n, s, ii, r, st, dx, zx);
  if (zx && n.p == 0.0f) {
    set_die(n, 1.0f);
    return;
  }
  if (!(n.die > 0.f)) untransform<D::pol>(c, n);
}

/* one non-linear block (mcramp.py:167-217): "multi" rounds of all
 * geometries then all scatters; no termination step. */
template <class D = NoDiff, bool EXT = true, bool MESH = true>
DI void block_nonlinear(const CompDev* comps, int first, int count, int multi, Nt& n,
                        uint32_t& ii, Rng& r, StatusDev* st, D* dx = nullptr) {
  Is s;
  is_reset(s);
  for (int e = 0; e < multi; ++e) {
    for (int j = first; j < first + count; ++j) {
      if (n.die > 0.f) break;
      const CompDev& c = comps[j];
      transform<D::pol>(c, n);
      if (intersect<MESH>(c, n, s, st)) ii = c.idx;
      untransform<D::pol>(c, n);
    }
    for (int j = first; j < first + count; ++j) {
      if (n.die > 0.f) break;
      const CompDev& c = comps[j];
      transform<D::pol>(c, n);
      if (ii == c.idx) scatter<D, EXT, MESH>(c, n, s, ii, r, st, dx);
      if (!(n.die > 0.f)) untransform<D::pol>(c, n);
    }
  }
}

/* ---- appending indices to a list shared by the whole grid -------------
 * (an atomic counter and its array).  Each warp gathers its entries in 64
 * words of shared memory (`stage`) and reserves list slots 32 at a time:
 * the counter takes one atomic per 32 entries, not one per warp pass.
 * `held` (warp-uniform, below 32 between calls) counts the gathered
 * entries; all 32 lanes call both functions.  Entries at or beyond `cap`
 * are dropped; the counter still counts them. */
__device__ __forceinline__ void warp_list_add(bool put, uint32_t v, uint32_t* stage, int& held,
                                              unsigned long long* count, uint32_t* list,
                                              int64_t cap) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, put);
  if (m == 0u) return;
  if (put) stage[held + __popc(m & ((1u << lane) - 1u))] = v;
  held += __popc(m);                                    /* at most 31 + 32 */
  if (held < 32) return;
  __syncwarp();
  unsigned long long at = 0;
  if (lane == 0) at = atomicAdd(count, 32ull);
  at = __shfl_sync(0xffffffffu, at, 0);
  if ((int64_t)(at + lane) < cap) list[at + lane] = stage[lane];
  held -= 32;
  const uint32_t rest = stage[32 + lane];
  __syncwarp();
  if (lane < held) stage[lane] = rest;
  __syncwarp();
}

__device__ __forceinline__ void warp_list_flush(const uint32_t* stage, int held,
                                                unsigned long long* count, uint32_t* list,
                                                int64_t cap) {
  if (held == 0) return;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  unsigned long long at = 0;
  if (lane == 0) at = atomicAdd(count, (unsigned long long)held);
  at = __shfl_sync(0xffffffffu, at, 0);
  if (lane < held && (int64_t)(at + lane) < cap) list[at + lane] = stage[lane];
}

#endif /* RAMP_DEVICE_CUH */
