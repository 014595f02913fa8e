/*
 * oracle.cpp — TEST INFRASTRUCTURE ONLY.  A CPU restatement of RAMP's
 * OpenCL kernels for the per-neutron chain, used by the parity tests and as
 * the timed CPU baseline.  Nothing in the product links or calls it.
 *
 * It keeps the reference's data layout and sequencing on purpose:
 *   - one 16-float record per neutron, one 8-float intersection record and
 *     one uint index per neutron, array-of-structs (NOTES:1-25,
 *     doc/writing/buffers.rst:1-88, mcramp/mcramp.py:386-401);
 *   - one pass over all neutrons per reference kernel launch: for every
 *     component of a linear block transform, intersect, terminate, scatter,
 *     untransform (mcramp.py:118-165); for non-linear blocks "multi" rounds
 *     of (transform, intersect, untransform) over all components followed
 *     by (transform, scatter, untransform) over all components
 *     (mcramp.py:167-217);
 *   - the reference RNG keying (mcramp/include/rand.h:4-21).
 * Each kernel function cites the .cl file it restates.  Arithmetic is FP32
 * throughout with unsuffixed literals taken as float (an OpenCL device
 * without cl_khr_fp64); built-ins map to ramp_gb300/csrc/rmath.h;
 * normalize(v) = v * (1/sqrt(dot(v,v))) (zero vectors unchanged),
 * length(v) = sqrt(dot(v,v)), dot sums left to right.  Where the reference
 * reads an uninitialised variable the value is taken as 0, and where it
 * would write or read outside a buffer the access is dropped and counted.
 *
 * Parity pins: the RNG (Threefry-4x32-20 and u01 conversion, rand.h) and
 * the supermirror reflectivity (include/ref.h) are checked against the
 * reference's own sources compiled with gcc (oracle/ref_pins), and every
 * kernel restated here against the reference's own .cl kernels compiled as
 * host C++ and run with the reference sequencing (oracle/refcl): with the
 * same math library the final records are bit-identical on every chain the
 * tests trace; the committed golden records (tests/golden/
 * refcl_records.npz) carry that pin where the reference is absent.
 *
 * Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (oracle/build.py)
 */
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <atomic>
#include <omp.h>

#include "../include/ramp.h"
#include "../ramp_gb300/csrc/rmath.h"
#include "../ramp_gb300/csrc/rconst.h"

namespace {

/* ---------------- float3 helpers (OpenCL vector built-ins) -------------- */
struct V3 { float x, y, z; };
inline V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mul(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 mulv(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(V3 a) { return sqrtf(dot(a, a)); }
inline V3 normalize(V3 a) {
  float d = dot(a, a);
  if (d == 0.0f) return a;
  float inv = 1.0f / sqrtf(d);
  return v3(a.x * inv, a.y * inv, a.z * inv);
}
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline bool all_eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

/* record accessors */
inline V3 npos(const float* n) { return v3(n[0], n[1], n[2]); }
inline V3 nvel(const float* n) { return v3(n[3], n[4], n[5]); }
inline V3 npol(const float* n) { return v3(n[6], n[7], n[8]); }
inline void set_pos(float* n, V3 v) { n[0] = v.x; n[1] = v.y; n[2] = v.z; }
inline void set_vel(float* n, V3 v) { n[3] = v.x; n[4] = v.y; n[5] = v.z; }
inline void set_pol(float* n, V3 v) { n[6] = v.x; n[7] = v.y; n[8] = v.z; }
inline V3 ipos1(const float* s) { return v3(s[0], s[1], s[2]); }
inline V3 ipos2(const float* s) { return v3(s[4], s[5], s[6]); }
inline void reset_isect(float* s) {
  s[0] = 0.0f; s[1] = 0.0f; s[2] = 0.0f; s[3] = RC_T_RESET;
  s[4] = 0.0f; s[5] = 0.0f; s[6] = 0.0f; s[7] = RC_T_RESET;
}
enum { P = 9, TOF = 10, SB = 11, SC = 12, SD = 13, SE = 14, DIE = 15 };

/* ---------------- Threefry-4x32-20 (Salmon et al., SC'11) -------------- */
inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

void threefry4x32_20(const uint32_t in[4], const uint32_t key[4], uint32_t out[4]) {
  static const int R[8][2] = {{10, 26}, {11, 21}, {13, 27}, {23, 5},
                              {6, 20}, {17, 11}, {25, 10}, {18, 20}};
  uint32_t ks[5];
  ks[4] = 0x1BD11BDAu;
  for (int i = 0; i < 4; ++i) { ks[i] = key[i]; ks[4] ^= key[i]; }
  uint32_t x0 = in[0] + ks[0], x1 = in[1] + ks[1], x2 = in[2] + ks[2], x3 = in[3] + ks[3];
  for (int r = 0; r < 20; ++r) {
    const int* rc = R[r % 8];
    if ((r & 1) == 0) {
      x0 += x1; x1 = rotl32(x1, rc[0]); x1 ^= x0;
      x2 += x3; x3 = rotl32(x3, rc[1]); x3 ^= x2;
    } else {
      x0 += x3; x3 = rotl32(x3, rc[0]); x3 ^= x0;
      x2 += x1; x1 = rotl32(x1, rc[1]); x1 ^= x2;
    }
    if ((r & 3) == 3) {
      uint32_t s = (uint32_t)(r / 4 + 1);
      x0 += ks[s % 5]; x1 += ks[(s + 1) % 5]; x2 += ks[(s + 2) % 5];
      x3 += ks[(s + 3) % 5] + s;
    }
  }
  out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* u01fixedpt_closed_closed_32_24 (Random123 u01fixedpt.h:137-140) */
inline float u01_cc_32_24(uint32_t i) {
  return (float)((i & 0x7fffffc0u) + (i & 0x40u)) * (1.0f / 2147483648.0f);
}

struct Keying {
  int mode;            /* 0 reference (rand.h), 1 native 4-words-per-block */
  uint32_t variant;
  uint32_t run_seed;
};

/* rand() — mcramp/include/rand.h:4-21.  Counter word 0 is (uint)sb, the
 * float counter converted with truncation (c.v[0] += counter, c.v[0]==0);
 * sb is incremented by one per draw. */
inline float o_rand(float* n, uint32_t tid, const Keying& kg) {
  uint32_t c = (uint32_t)n[SB];
  uint32_t out[4];
  float u;
  if (kg.mode == 0) {
    const uint32_t key[4] = {tid, 0xdecafbadu, 0xfacebeadu, 0x12345678u};
    const uint32_t ctr[4] = {c, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
    threefry4x32_20(ctr, key, out);
    u = u01_cc_32_24(out[0]);
  } else {
    const uint32_t key[4] = {tid, kg.variant, kg.run_seed, 0x12345678u};
    const uint32_t ctr[4] = {c >> 2, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
    threefry4x32_20(ctr, key, out);
    u = u01_cc_32_24(out[c & 3u]);
  }
  n[SB] += 1.0f;
  return u;
}

/* ---------------- frame rotation — mcramp/include/geom.h:21-87 ---------- */
struct Rot { float r00, r01, r02, r10, r11, r12, r20, r21, r22; };
inline Rot rot_matrix(const float* rot) {
  float x_a = rot[0], y_a = rot[1], z_a = rot[2];
  float cx = rm_cosf(x_a), sx = rm_sinf(x_a);
  float cy = rm_cosf(y_a), sy = rm_sinf(y_a);
  float cz = rm_cosf(z_a), sz = rm_sinf(z_a);
  Rot R;
  R.r00 = cy * cz;
  R.r01 = -cx * sz + sx * sy * cz;
  R.r02 = sx * sz + cx * sy * cz;
  R.r10 = cy * sz;
  R.r11 = cx * cz + sx * sy * sz;
  R.r12 = -sx * cz + cx * sy * sz;
  R.r20 = -sy;
  R.r21 = sx * cy;
  R.r22 = cx * cy;
  return R;
}
inline V3 frame_rotate(V3 v, const float* rot) {
  Rot R = rot_matrix(rot);
  return v3(dot(v3(R.r00, R.r01, R.r02), v), dot(v3(R.r10, R.r11, R.r12), v),
            dot(v3(R.r20, R.r21, R.r22), v));
}
inline V3 frame_derotate(V3 v, const float* rot) {
  Rot R = rot_matrix(rot);
  return v3(dot(v3(R.r00, R.r10, R.r20), v), dot(v3(R.r01, R.r11, R.r21), v),
            dot(v3(R.r02, R.r12, R.r22), v));
}

/* rotate_about_axis — mcramp/include/geom.h:1-19 */
inline V3 rotate_about_axis(float angle, V3 a, V3 v) {
  float c = rm_cosf(angle), s = rm_sinf(angle);
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

/* reflectivity_func — mcramp/include/ref.h:3-53 (beta taken as 0 when the
 * m-parametrisation does not set it) */
float reflectivity(float q, float R0, float Qc, float alpha, float m, float W) {
  float beta = 0.0f, arg, R = 0.0f;
  if (W == 0.0f && alpha == 0.0f) {
    m = m * 0.9853f + 0.1978f;
    W = -0.0002f * m + 0.0022f;
    alpha = 0.2304f * m + 5.0944f;
    beta = -7.6251f * m + 68.1137f;
    if (m <= 3) { alpha = m; beta = 0; }
  }
  arg = W > 0 ? (q - m * Qc) / W : 11;
  if (arg > 10 || m <= 0 || Qc <= 0 || R0 <= 0) { R = 0.0f; return R; }
  if (m < 1) { Qc *= m; m = 1; }
  if (q <= Qc) { R = R0; return R; }
  R = R0 * 0.5f * (1 - rm_tanhf(arg)) * (1 - alpha * (q - Qc) + beta * (q - Qc) * (q - Qc));
  return R;
}

/* ---------------- shared context for a pass ----------------------------- */
struct Ctx {
  float* neutrons;     /* [n][16] */
  float* isect;        /* [n][8]  */
  uint32_t* iidx;      /* [n]     */
  int64_t n;
  Keying kg;
  uint32_t tid_base;   /* global id of record 0 */
  std::atomic<uint64_t>* oob;
  std::atomic<uint32_t>* flags;
};

/* Tally addition.  The GPU's float atomics flush subnormal operands to
 * zero (the reference's CAS-loop add leaves this to the OpenCL device), so
 * terms are flushed the same way here. */
inline float ftz(float x) { return fabsf(x) < 1.17549435e-38f ? copysignf(0.0f, x) : x; }
inline void atomic_add_f(float* addr, float v) {
  v = ftz(v);
#pragma omp atomic
  *addr += v;
}

/* ---------------- moderators ------------------------------------------- */
/* generate_neutrons — mcramp/moderator/flat_mod.cl:4-50 */
void gen_flat(const Ctx& c, const RampSource& s, int32_t num_sim, int32_t seed) {
  const float mdx = s.p[0], mdy = s.p[1], tdx = s.p[2], tdy = s.p[3];
  const float target_dist = s.p[4], E_min = s.p[5], E_max = s.p[6];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    uint32_t tid = c.tid_base + (uint32_t)i;
    float old_sb = n[SB];
    for (int k = 0; k < 16; ++k) n[k] = 0.0f;
    n[SB] = (float)seed + old_sb;
    float E_range = (E_max - E_min);
    float E_val = E_min + E_range * o_rand(n, tid, c.kg);
    n[P] = 1.0f / (float)num_sim;
    n[0] = mdx * (0.5f - o_rand(n, tid, c.kg));
    n[1] = mdy * (0.5f - o_rand(n, tid, c.kg));
    n[2] = 0.0f;
    float vel = RC_SE2V * sqrtf(E_val);
    float Dx = tdx * (0.5f - o_rand(n, tid, c.kg)) - n[0];
    float Dy = tdy * (0.5f - o_rand(n, tid, c.kg)) - n[1];
    set_vel(n, mul(vel, normalize(v3(Dx, Dy, target_dist))));
    float theta = 2 * RC_PI * o_rand(n, tid, c.kg);
    float phi = rm_acosf(1 - 2 * o_rand(n, tid, c.kg));
    n[6] = rm_sinf(phi) * rm_cosf(theta);
    n[7] = rm_sinf(phi) * rm_sinf(theta);
    n[8] = rm_cosf(phi);
    n[DIE] = 0.0f;
    reset_isect(c.isect + 8 * i);
  }
}

/* maxwell_energy_distn — mcramp/moderator/cont_mod.cl:4-9; pow(x, 1.5) is
 * evaluated as x*sqrt(x) */
inline float maxwell(float E, float T) {
  float rootE = sqrtf(E);
  float overKT = 1.0f / (RC_K_B * T);
  return 2.0f * rootE / sqrtf(RC_PI) * (overKT * sqrtf(overKT)) * rm_expf(-E * overKT);
}

/* generate_neutrons — mcramp/moderator/cont_mod.cl:11-72 */
void gen_cont(const Ctx& c, const RampSource& s, int32_t num_sim, int32_t seed) {
  const float mdx = s.p[0], mdy = s.p[1], tdx = s.p[2], tdy = s.p[3];
  const float target_dist = s.p[4], E_min = s.p[5], E_max = s.p[6];
  const float T1 = s.p[7], I1 = s.p[8], T2 = s.p[9], I2 = s.p[10], T3 = s.p[11], I3 = s.p[12];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    uint32_t tid = c.tid_base + (uint32_t)i;
    float old_sb = n[SB];
    for (int k = 0; k < 16; ++k) n[k] = 0.0f;
    n[SB] = (float)seed + old_sb;
    float E_range = (E_max - E_min);
    float E_val = E_min + E_range * o_rand(n, tid, c.kg);
    float E_J = RC_EV_J * E_val;
    float d1 = maxwell(RC_K_B * T1, T1);
    float d2 = maxwell(RC_K_B * T2, T2);
    float d3 = maxwell(RC_K_B * T3, T3);
    float M = I1 * maxwell(E_J, T1) / d1;
    M += I2 * maxwell(E_J, T2) / d2;
    M += I3 * maxwell(E_J, T3) / d3;
    n[P] = M / (float)num_sim;
    n[0] = mdx * (0.5f - o_rand(n, tid, c.kg));
    n[1] = mdy * (0.5f - o_rand(n, tid, c.kg));
    n[2] = 0.0f;
    float vel = RC_SE2V * sqrtf(E_val);
    float Dx = tdx * (0.5f - o_rand(n, tid, c.kg)) - n[0];
    float Dy = tdy * (0.5f - o_rand(n, tid, c.kg)) - n[1];
    set_vel(n, mul(vel, normalize(v3(Dx, Dy, target_dist))));
    float theta = 2 * RC_PI * o_rand(n, tid, c.kg);
    float phi = rm_acosf(1 - 2 * o_rand(n, tid, c.kg));
    n[6] = rm_sinf(phi) * rm_cosf(theta);
    n[7] = rm_sinf(phi) * rm_sinf(theta);
    n[8] = rm_cosf(phi);
    n[DIE] = 0.0f;
    reset_isect(c.isect + 8 * i);
  }
}

/* find_closest_in_cdf — mcramp/moderator/isis_mod.cl:4-13, a linear scan;
 * entries past the table read as 0 (the reference passes n_t * n_e, one
 * energy row more than the flux table holds) */
inline float isis_at(const float* t, int64_t len, int64_t i) {
  return (i >= 0 && i < len) ? t[i] : 0.0f;
}
inline int isis_cdf(const float* t, int64_t len, int64_t scan, float val) {
  for (int64_t i = 0; i < scan; i++)
    if ((isis_at(t, len, i) - val) > 0.0f) return (int)(i - 1);
  return 0;
}

/* generate_neutrons — mcramp/moderator/isis_mod.cl:15-104 */
void gen_isis(const Ctx& c, const RampSource& s, int32_t num_sim, int32_t seed) {
  const float mdx = s.p[0], mdy = s.p[1], tdx = s.p[2], tdy = s.p[3];
  const float target_dist = s.p[4], str_area = s.p[13], total = s.p[14];
  const float* flux = s.table[0];
  const float* tb = s.table[1];
  const float* eb = s.table[2];
  const float* ei = s.table[3];
  const int64_t nflux = s.table_len[0];
  const int nt = (int)s.table_len[1], ne = (int)s.table_len[2];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    uint32_t tid = c.tid_base + (uint32_t)i;
    float old_sb = n[SB];
    for (int k = 0; k < 16; ++k) n[k] = 0.0f;
    n[SB] = (float)seed + old_sb;
    float deviate = total * o_rand(n, tid, c.kg);
    int idx = isis_cdf(flux, nflux, (int64_t)nt * ne, deviate);
    int Epnt = isis_cdf(ei, ne, ne, deviate);
    int Tpnt = (int)fmodf((float)idx, (float)nt);
    if (Tpnt >= nt - 1) Tpnt -= 1;
    float time_val = isis_at(tb, nt, Tpnt);
    float time_range = isis_at(tb, nt, Tpnt + 1) - isis_at(tb, nt, Tpnt);
    float time_spread = isis_at(flux, nflux, (int64_t)Epnt * nt + Tpnt + 1) -
                        isis_at(flux, nflux, (int64_t)Epnt * nt + Tpnt);
    float R = deviate - isis_at(flux, nflux, (int64_t)Epnt * nt + Tpnt);
    R /= time_spread;
    time_val += time_range * R;
    float ener_spread = isis_at(ei, ne, Epnt + 1) - isis_at(ei, ne, Epnt);
    int i0 = (Epnt > 3) ? Epnt - 3 : 0;
    int i1 = ((ne - Epnt - 1) > 3) ? Epnt + 3 : (ne - 1);
    deviate = isis_at(ei, ne, Epnt) + ener_spread * o_rand(n, tid, c.kg);
    float accumulator = 0.0f;
    for (int a = i0; a <= i1; a++) {
      float Pj = 1.0f;
      for (int b = i0; b <= i1; b++)
        if (b != a) Pj *= (deviate - isis_at(ei, ne, b)) / (isis_at(ei, ne, a) - isis_at(ei, ne, b));
      Pj *= isis_at(eb, ne, a);
      accumulator += Pj;
    }
    float ener_val = accumulator;
    n[0] = mdx * (0.5f - o_rand(n, tid, c.kg));
    n[1] = mdy * (0.5f - o_rand(n, tid, c.kg));
    n[2] = 0.0f;
    float vel = RC_SE2V * sqrtf(ener_val);
    float Dx = tdx * (0.5f - o_rand(n, tid, c.kg)) - n[0];
    float Dy = tdy * (0.5f - o_rand(n, tid, c.kg)) - n[1];
    set_vel(n, mul(vel, normalize(v3(Dx, Dy, target_dist))));
    float theta = 2 * RC_PI * o_rand(n, tid, c.kg);
    float phi = rm_acosf(1 - 2 * o_rand(n, tid, c.kg));
    n[6] = rm_sinf(phi) * rm_cosf(theta);
    n[7] = rm_sinf(phi) * rm_sinf(theta);
    n[8] = rm_cosf(phi);
    n[P] = str_area * total * 6.2415093e+12f / (float)num_sim;
    n[TOF] = time_val;
    n[DIE] = 0.0f;
    reset_isect(c.isect + 8 * i);
  }
}

/* ---------------- frame transform & termination ------------------------- */
/* transform — mcramp/scat/frametransform.cl:4-23 */
void transform(const Ctx& c, const RampComp& k) {
  V3 cp = v3(k.pos[0], k.pos[1], k.pos[2]);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    if (n[DIE] > 0.f) continue;
    set_pos(n, sub(npos(n), cp));
    set_pos(n, frame_derotate(npos(n), k.rot));
    set_vel(n, frame_derotate(nvel(n), k.rot));
    set_pol(n, frame_derotate(npol(n), k.rot));
  }
}

/* untransform — mcramp/scat/frametransform.cl:25-42 */
void untransform(const Ctx& c, const RampComp& k) {
  V3 cp = v3(k.pos[0], k.pos[1], k.pos[2]);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    if (n[DIE] > 0.f) continue;
    set_pos(n, frame_rotate(npos(n), k.rot));
    set_pos(n, add(npos(n), cp));
    set_vel(n, frame_rotate(nvel(n), k.rot));
    set_pol(n, frame_rotate(npol(n), k.rot));
  }
}

/* terminate — mcramp/scat/terminator.cl:3-21 */
void terminate(const Ctx& c, const RampComp& k) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    const float* s = c.isect + 8 * i;
    if (n[DIE] > 0.0f) continue;
    if (length(ipos2(s)) == 0.0f && k.restore == 0) n[DIE] = 1.f;
  }
}

/* ---------------- geometry kernels ------------------------------------- */
/* intersect_plane — mcramp/geom/plane.cl:3-52 */
void g_plane(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float width = k.gp[0], height = k.gp[1];
  const int orientation = k.gi[0];
  V3 vel = nvel(n), pos = npos(n);
  float t = 0.0f, x = 0.0f, y = 0.0f;
  if (orientation == 0) {
    t = (-pos.z) / vel.z; x = pos.x + t * vel.x; y = pos.y + t * vel.y;
  } else if (orientation == 1) {
    t = (-pos.x) / vel.x; x = pos.z + t * vel.z; y = pos.y + t * vel.y;
  }
  if ((fabsf(x) < width / 2.0f) && (fabsf(y) < height / 2.0f) && t < s[3] && t < s[7] &&
      t > 0.0f && dot(vel, v3(0.0f, 0.0f, 1.0f)) > 0.f) {
    V3 h = add(pos, mul(t, vel));
    s[0] = h.x; s[1] = h.y; s[2] = h.z;
    s[4] = h.x; s[5] = h.y; s[6] = h.z;
    s[3] = t; s[7] = t;
    *iidx = k.idx;
  }
}

/* intersect — mcramp/geom/cylinder_ext.cl:3-53 (theta2 is unused there) */
void g_cyl_ext(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float radius = k.gp[0], height = k.gp[1];
  float ppx = n[0], ppz = n[2], pvx = n[3], pvz = n[5];
  float a = pvx * pvx + pvz * pvz;
  float b = 2.0f * (ppx * pvx + ppz * pvz);
  float cc = (ppx * ppx + ppz * ppz) - radius * radius;
  float quotient = b * b - 4.0f * a * cc;
  float t1 = (-b - sqrtf(quotient)) / (2.f * a);
  float t2 = (-b + sqrtf(quotient)) / (2.f * a);
  float yt2 = n[1] + t2 * n[4];
  if ((quotient > 0.0f) && ((-height / 2.0f) < yt2) && (yt2 < (height / 2))) {
    if (t1 < s[3] && t1 > 0.0f && t2 > 0.0f) {
      V3 p1 = add(npos(n), mul(t1, nvel(n)));
      s[0] = p1.x; s[1] = p1.y; s[2] = p1.z; s[3] = t1;
      *iidx = k.idx;
      V3 p2 = add(npos(n), mul(t2, nvel(n)));
      s[4] = p2.x; s[5] = p2.y; s[6] = p2.z; s[7] = t2;
    }
  }
}

/* intersect_banana — mcramp/geom/banana.cl:3-55.  The angular window is the
 * C chained comparison (mintheta < theta2) < maxtheta (banana.cl:38). */
void g_banana(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float radius = k.gp[0], height = k.gp[1], mintheta = k.gp[2], maxtheta = k.gp[3];
  float ppx = n[0], ppz = n[2], pvx = n[3], pvz = n[5];
  float a = pvx * pvx + pvz * pvz;
  float b = 2.0f * (ppx * pvx + ppz * pvz);
  float cc = (ppx * ppx + ppz * ppz) - radius * radius;
  float quotient = b * b - 4.0f * a * cc;
  float t1 = (-b - sqrtf(quotient)) / (2.f * a);
  float t2 = (-b + sqrtf(quotient)) / (2.f * a);
  /* theta2 = acos(dot(normalize(plane_pos + t2*plane_vel), (0,1))) */
  float hx = ppx + t2 * pvx, hz = ppz + t2 * pvz;
  float d2 = hx * hx + hz * hz;
  float nz = hz;
  if (d2 != 0.0f) { float inv = 1.0f / sqrtf(d2); nz = hz * inv; hx = hx * inv; }
  float theta2 = rm_acosf(hx * 0.0f + nz * 1.0f);
  float window = (float)(mintheta < theta2);
  float yt2 = n[1] + t2 * n[4];
  if ((quotient > 0.0f) && ((-height / 2.0f) < yt2) && (yt2 < (height / 2)) && (window < maxtheta)) {
    if (t2 < s[3] && t1 < 0.0f && t2 > 0.0f) {
      V3 p1 = add(npos(n), mul(t1, nvel(n)));
      s[0] = p1.x; s[1] = p1.y; s[2] = p1.z; s[3] = t1;
      *iidx = k.idx;
      V3 p2 = add(npos(n), mul(t2, nvel(n)));
      s[4] = p2.x; s[5] = p2.y; s[6] = p2.z; s[7] = t2;
    }
  }
}

/* intersect_sphere — mcramp/geom/sphere.cl:3-42 */
void g_sphere(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  V3 pos = npos(n), vel = nvel(n);
  float r = k.gp[0];
  float a = dot(vel, vel);
  float b = 2.0f * (dot(vel, pos));
  float cc = dot(pos, pos) - r * r;
  float quotient = b * b - 4.0f * a * cc;
  if (quotient > 0.0f) {
    float d1 = (-b - sqrtf(quotient)) / (2.f * a);
    float d2 = (-b + sqrtf(quotient)) / (2.f * a);
    if (d1 < s[3] && d1 > 0.f) {
      V3 p1 = add(pos, mul(d1, vel));
      s[0] = p1.x; s[1] = p1.y; s[2] = p1.z; s[3] = d1;
      *iidx = k.idx;
      V3 p2 = add(pos, mul(d2, vel));
      s[4] = p2.x; s[5] = p2.y; s[6] = p2.z; s[7] = d2;
    }
  }
}

/* intersect_sphere — mcramp/geom/sphere_int.cl:3-41 */
void g_sphere_int(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  V3 pos = npos(n), vel = nvel(n);
  float r = k.gp[0];
  float a = dot(vel, vel);
  float b = 2.0f * (dot(vel, pos));
  float cc = dot(pos, pos) - r * r;
  float quotient = b * b - 4.0f * a * cc;
  if (quotient > 0.0f) {
    float d1 = (-b - sqrtf(quotient)) / (2.f * a);
    float d2 = (-b + sqrtf(quotient)) / (2.f * a);
    if (d1 < 0.0f && d2 < s[3]) {
      V3 p2 = add(pos, mul(d2, vel));
      s[0] = p2.x; s[1] = p2.y; s[2] = p2.z; s[3] = d2;
      *iidx = k.idx;
      s[4] = p2.x; s[5] = p2.y; s[6] = p2.z; s[7] = d2;
    }
  }
}

/* intersect_box — mcramp/geom/box.cl:3-53 (no earliest-hit comparison).
 * The kernel never loads the intersection record (box.cl:10) and stores
 * its local copy back on a miss too (:52): a store of an undefined value,
 * which an optimising OpenCL compiler removes, so the record is kept. */
void g_box(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  V3 pos = npos(n), vel = nvel(n);
  V3 A = v3(-k.gp[0] / 2.0f, -k.gp[1] / 2.0f, -k.gp[2] / 2.0f);
  V3 B = v3(k.gp[0] / 2.0f, k.gp[1] / 2.0f, k.gp[2] / 2.0f);
  V3 dA = sub(A, pos), dB = sub(B, pos);
  float t1 = dA.x / vel.x, t2 = dB.x / vel.x, t3 = dA.y / vel.y;
  float t4 = dB.y / vel.y, t5 = dA.z / vel.z, t6 = dB.z / vel.z;
  float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
  float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
  if (tmax < 0.0f) {
  } else if (tmin > tmax) {
  } else {
    V3 p1 = add(pos, mul(tmin, vel)), p2 = add(pos, mul(tmax, vel));
    s[0] = p1.x; s[1] = p1.y; s[2] = p1.z; s[3] = tmin;
    s[4] = p2.x; s[5] = p2.y; s[6] = p2.z; s[7] = tmax;
    *iidx = k.idx;
  }
}

/* arm — mcramp/geom/arm.cl:3-21 */
void g_arm(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  (void)n;
  s[4] = 1.0f; s[5] = 1.0f; s[6] = 1.0f;
  *iidx = k.idx;
}

/* Watertight ray/triangle crossing (Woop, Benthin, Wald: "Watertight
 * Ray/Triangle Intersection", JCGT 2(1), 2013) used for SAttenuate's chord:
 * edge functions of a shared edge are exact negations of each other, so a
 * ray through an edge crosses exactly one of its two faces; exact zeros are
 * re-evaluated in double.  Returns the ray parameter t (NaN: no crossing).
 * kx, ky, kz and Sx, Sy, Sz are the per-ray shear of the method. */
struct Shear { int kx, ky, kz; float Sx, Sy, Sz; };
Shear make_shear(V3 d) {
  float ad[3] = {fabsf(d.x), fabsf(d.y), fabsf(d.z)};
  float dd[3] = {d.x, d.y, d.z};
  Shear S;
  S.kz = (ad[0] > ad[1]) ? ((ad[0] > ad[2]) ? 0 : 2) : ((ad[1] > ad[2]) ? 1 : 2);
  S.kx = (S.kz + 1) % 3; S.ky = (S.kx + 1) % 3;
  if (dd[S.kz] < 0.0f) { int t = S.kx; S.kx = S.ky; S.ky = t; }
  S.Sx = dd[S.kx] / dd[S.kz]; S.Sy = dd[S.ky] / dd[S.kz]; S.Sz = 1.0f / dd[S.kz];
  return S;
}
float watertight_t(const Shear& S, V3 org, V3 v0, V3 v1, V3 v2) {
  float A[3] = {v0.x - org.x, v0.y - org.y, v0.z - org.z};
  float B[3] = {v1.x - org.x, v1.y - org.y, v1.z - org.z};
  float C[3] = {v2.x - org.x, v2.y - org.y, v2.z - org.z};
  float Ax = A[S.kx] - S.Sx * A[S.kz], Ay = A[S.ky] - S.Sy * A[S.kz];
  float Bx = B[S.kx] - S.Sx * B[S.kz], By = B[S.ky] - S.Sy * B[S.kz];
  float Cx = C[S.kx] - S.Sx * C[S.kz], Cy = C[S.ky] - S.Sy * C[S.kz];
  float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return NAN;
  float det = U + V + W;
  if (det == 0.0f) return NAN;
  float Az = S.Sz * A[S.kz], Bz = S.Sz * B[S.kz], Cz = S.Sz * C[S.kz];
  float T = U * Az + V * Bz + W * Cz;
  return T / det;
}

/* intersect — mcramp/geom/mesh.cl:3-129 (brute force over all triangles).
 * With an SAttenuate scatter the chord time through the mesh is kept in the
 * record's lane sd: the sum over watertight crossings with t > eps of +t
 * (leaving, n.v > 0) or -t (entering), i.e. the winding-number weighted time
 * inside the surface, clamped at 0. */
void g_mesh(const Ctx&, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float* pts = k.table[0];
  const uint32_t num_tri = (uint32_t)(k.table_len[0] / 9);
  const int interior = k.gi[0];
  V3 pos = npos(n), vel = nvel(n);
  V3 ll = v3(k.gp[0], k.gp[2], k.gp[4]), ur = v3(k.gp[1], k.gp[3], k.gp[5]);
  V3 dA = sub(ll, pos), dB = sub(ur, pos);
  float t1 = dA.x / vel.x, t2 = dB.x / vel.x, t3 = dA.y / vel.y;
  float t4 = dB.y / vel.y, t5 = dA.z / vel.z, t6 = dB.z / vel.z;
  float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
  float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
  if (tmax < 0.0f || tmin > tmax) return;
  const float eps = 0.000000001f;
  uint32_t num_intersections = 0;
  float out[8] = {0.0f, 0.0f, 0.0f, 1e8f, 0.0f, 0.0f, 0.0f, 1e8f};
  const bool want_chord = (k.scat == RAMP_S_ATTENUATE);
  Shear S = make_shear(vel);
  double chord = 0.0;
  for (uint32_t i = 0; i < num_tri; ++i) {
    const float* p = pts + 9 * (size_t)i;
    V3 v0 = v3(p[0], p[1], p[2]), v1 = v3(p[3], p[4], p[5]), v2 = v3(p[6], p[7], p[8]);
    V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    V3 h = cross(vel, e2);
    float a = dot(e1, h);
    if (fabsf(a) < eps) continue;
    float f = 1.0f / a;
    V3 sv = sub(pos, v0);
    float u = f * dot(sv, h);
    if (u < 0.0f || u > 1.0f) continue;
    V3 q = cross(sv, e1);
    float v = f * dot(vel, q);
    if (v < 0.0f || u + v > 1.0f) continue;
    float t = f * dot(e2, q);
    if (t > eps) num_intersections++;
    V3 nrm = cross(e1, e2);
    float nv = dot(nrm, vel);
    if ((t > eps) && (t < out[3]) && (nv < 0)) {
      V3 hp = add(pos, mulv(vel, t));
      out[0] = hp.x; out[1] = hp.y; out[2] = hp.z; out[3] = t;
    }
    if ((t > eps) && (t < out[7]) && (nv > 0)) {
      V3 hp = add(pos, mulv(vel, t));
      out[4] = hp.x; out[5] = hp.y; out[6] = hp.z; out[7] = t;
    }
  }
  if (want_chord) {
    for (uint32_t i = 0; i < num_tri; ++i) {
      const float* p = pts + 9 * (size_t)i;
      V3 v0 = v3(p[0], p[1], p[2]), v1 = v3(p[3], p[4], p[5]), v2 = v3(p[6], p[7], p[8]);
      float tw = watertight_t(S, pos, v0, v1, v2);
      if (!(tw > eps)) continue;
      float nv = dot(cross(sub(v1, v0), sub(v2, v0)), vel);
      if (nv > 0) chord += (double)tw;
      else if (nv < 0) chord -= (double)tw;
    }
  }
  if ((interior == 1) && (num_intersections % 2 == 1)) {
    for (int j = 0; j < 4; ++j) out[4 + j] = out[j];
  } else if ((interior == 1) && (num_intersections % 2 == 0)) {
    return;
  }
  if (out[3] < s[3]) {
    for (int j = 0; j < 8; ++j) s[j] = out[j];
    *iidx = k.idx;
    if (want_chord) n[SD] = chord > 0.0 ? (float)chord : 0.0f;
  }
}

void intersect(const Ctx& c, const RampComp& k) {
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    float* s = c.isect + 8 * i;
    if (n[DIE] > 0.f) continue;
    switch (k.geom) {
      case RAMP_G_PLANE: g_plane(n, s, c.iidx + i, k); break;
      case RAMP_G_CYL_EXT: g_cyl_ext(n, s, c.iidx + i, k); break;
      case RAMP_G_BANANA: g_banana(n, s, c.iidx + i, k); break;
      case RAMP_G_SPHERE: g_sphere(n, s, c.iidx + i, k); break;
      case RAMP_G_SPHERE_INT: g_sphere_int(n, s, c.iidx + i, k); break;
      case RAMP_G_BOX: g_box(n, s, c.iidx + i, k); break;
      case RAMP_G_ARM: g_arm(n, s, c.iidx + i, k); break;
      case RAMP_G_MESH: g_mesh(c, n, s, c.iidx + i, k); break;
      default: break;
    }
  }
}

/* ---------------- scattering kernels ------------------------------------ */
inline void finish(float* n, float* s, uint32_t* iidx, const RampComp& k) {
  *iidx = 0;
  n[SC] = (float)k.idx;
  reset_isect(s);
}

/* arm — mcramp/scat/arm.cl:3-29 (leaves iidx and prevcomp as they are) */
void s_arm(const Ctx&, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  (void)n;
  *iidx = k.idx;
  reset_isect(s);
}

/* beamstop — mcramp/scat/beamstop.cl:3-32 */
void s_beamstop(const Ctx&, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  n[DIE] = 1.0f;
  finish(n, s, iidx, k);
}

/* counter — mcramp/scat/counter.cl:18-49 */
void s_counter(const Ctx&, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  if (k.tally) atomic_add_f(&k.tally[0], n[P]);
  n[SE] = 1.0f;
  finish(n, s, iidx, k);
}

/* guide_scatter — mcramp/scat/guide.cl:9-149 (FP32).  The loop index i is
 * reset on every bounce (guide.cl:66), so max_bounces ends the loop only
 * when it is below 6; a hard cap kills neutrons that would bounce forever. */
void s_guide(const Ctx& c, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float w1 = k.sp[0], h1 = k.sp[1], w2 = k.sp[2], h2 = k.sp[3], l = k.sp[4];
  const float R0 = k.sp[5], Qc = k.sp[6], alpha = k.sp[7], m = k.sp[8], W = k.sp[9];
  const uint32_t max_bounces = (uint32_t)k.si[0];
  set_pos(n, ipos2(s));
  n[TOF] += s[7];
  float t1, t2, av, ah, bv, bh, cv1, cv2, ch1, ch2, d = 0, ww, hh, whalf, hhalf;
  float vdotn_v1, vdotn_v2, vdotn_h1, vdotn_h2, q = 0, nlen2, refl;
  uint32_t i = 0;
  ww = 0.5f * (w2 - w1); hh = 0.5f * (h2 - h1);
  whalf = 0.5f * w1; hhalf = 0.5f * h1;
  int guard = 0;
  while (i < max_bounces) {
    if (++guard > RC_GUIDE_HARD_CAP) {
      n[DIE] = 1.0f;
      c.flags->fetch_or(RAMP_F_GUIDE_CAP);
      break;
    }
    V3 pos = npos(n), vel = nvel(n);
    av = l * vel.x; bv = ww * vel.z;
    ah = l * vel.y; bh = hh * vel.z;
    vdotn_v1 = bv + av; vdotn_v2 = bv - av;
    vdotn_h1 = bh + ah; vdotn_h2 = bh - ah;
    cv1 = -whalf * l - pos.z * ww; cv2 = pos.x * l;
    ch1 = -hhalf * l - pos.z * hh; ch2 = pos.y * l;
    t1 = (l - pos.z) / vel.z;
    i = 0;
    if (vdotn_v1 < 0.0f && (t2 = (cv1 - cv2) / vdotn_v1) < t1) { t1 = t2; i = 1; }
    if (vdotn_v2 < 0.0f && (t2 = (cv1 + cv2) / vdotn_v2) < t1) { t1 = t2; i = 2; }
    if (vdotn_h1 < 0.0f && (t2 = (ch1 - ch2) / vdotn_h1) < t1) { t1 = t2; i = 3; }
    if (vdotn_h2 < 0.0f && (t2 = (ch1 + ch2) / vdotn_h2) < t1) { t1 = t2; i = 4; }
    if (i == 0) break;
    set_pos(n, add(npos(n), mul(t1, vel)));
    n[TOF] += t1;
    switch (i) {
      case 1:
        nlen2 = l * l + ww * ww;
        q = RC_V2K * (-2.0f) * vdotn_v1 / sqrtf(nlen2);
        d = 2.0f * vdotn_v1 / nlen2;
        n[3] = n[3] - d * l; n[5] = n[5] - d * ww;
        break;
      case 2:
        nlen2 = l * l + ww * ww;
        q = RC_V2K * (-2.0f) * vdotn_v2 / sqrtf(nlen2);
        d = 2.0f * vdotn_v2 / nlen2;
        n[3] = n[3] + d * l; n[5] = n[5] - d * ww;
        break;
      case 3:
        nlen2 = l * l + hh * hh;
        q = RC_V2K * (-2.0f) * vdotn_h1 / sqrtf(nlen2);
        d = 2.0f * vdotn_h1 / nlen2;
        n[4] = n[4] - d * l; n[5] = n[5] - d * hh;
        break;
      case 4:
        nlen2 = l * l + hh * hh;
        q = RC_V2K * (-2.0f) * vdotn_h2 / sqrtf(nlen2);
        d = 2.0f * vdotn_h2 / nlen2;
        n[4] = n[4] + d * l; n[5] = n[5] - d * hh;
        break;
    }
    refl = reflectivity(q, R0, Qc, alpha, m, W);
    n[P] *= refl;
    if (refl < 1e-12f || refl > 1.0f) n[P] = 0.0f;
    i++;
  }
  if (i >= max_bounces) n[DIE] = 1.0f;
  *iidx = 0;
  n[SC] = (float)k.idx;
  reset_isect(s);
}

/* chopper — mcramp/scat/chopper.cl:4-59 */
void s_chopper(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float slit_width = k.sp[0], radius = k.sp[1], freq = k.sp[2], phase = k.sp[3];
  const float jitter = k.sp[4];
  const uint32_t n_slits = (uint32_t)k.si[0];
  uint32_t tid = c.tid_base + (uint32_t)i;
  set_pos(n, ipos2(s));
  n[TOF] += s[7];
  float Tg = 2.0f * RC_PI / (float)n_slits;
  float pha_error = jitter * 2.0f * (o_rand(n, tid, c.kg) - 0.5f);
  float thi_chop = freq * (n[TOF] - fabsf(phase)) + pha_error;
  float thi_neut = rm_atan2f(n[0], n[1] + radius);
  float thi_diff = fabsf(thi_chop - thi_neut);
  float ang_diff = fmodf(thi_diff, Tg);
  if (fabsf(ang_diff - Tg) < ang_diff) ang_diff = fabsf(ang_diff - Tg);
  float width = rm_atan2f(slit_width, n[1] + radius);
  if (ang_diff > width / 2.0f) n[DIE] = 1.0f;
  finish(n, s, iidx, k);
}

/* sample_distn — mcramp/scat/isotropic.cl:5-73 (omega, Q, w_index start at
 * 0; a table index past the end is never read: the scans stop at the
 * table lengths) */
inline void sample_distn(float* n, uint32_t tid, const Keying& kg, const float* q,
                         const float* w, const float* pw_cdf, const float* pq_cdf,
                         uint32_t qsamples, uint32_t wsamples, float* omega_o, float* Q_o) {
  float mindiff, u, v, omega = 0.0f, Q = 0.0f;
  uint32_t w_index = 0;
  u = o_rand(n, tid, kg);
  v = o_rand(n, tid, kg);
  mindiff = 1.f;
  for (uint32_t i = 0; i < wsamples; i++) {
    if (pw_cdf[i] == 1.f) break;
    if (fabsf(pw_cdf[i] - v) < mindiff) {
      mindiff = fabsf(pw_cdf[i] - v);
      float lo = (i > 0 ? w[i - 1] : 0.0f);
      omega = lo + (o_rand(n, tid, kg)) * (w[i] - lo);
      w_index = i;
    }
  }
  mindiff = 1.f;
  for (uint32_t i = 0; i < qsamples; i++) {
    if (pq_cdf[w_index * qsamples + i] == 1.f) break;
    if (fabsf(pq_cdf[w_index * qsamples + i] - u) < mindiff) {
      mindiff = fabsf(pq_cdf[w_index * qsamples + i] - u);
      float lo = (i > 0 ? q[i - 1] : 0.0f);
      Q = lo + (o_rand(n, tid, kg)) * (q[i] - lo);
    }
  }
  *omega_o = omega;
  *Q_o = Q;
}

/* isotropic_scatter — mcramp/scat/isotropic.cl:75-322.  Tables per
 * channel c (0 coh, 1 inc, 2 mag): table[4c..4c+3] = q, w, pw_cdf, pq_cdf;
 * sp[1+3c..3+3c] = rho, sigma_abs, sigma_scat; si[1+2c], si[2+2c] =
 * qsamples, wsamples; sp[0] temperature; si[0] transmit. */
void s_isotropic(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  uint32_t tid = c.tid_base + (uint32_t)i;
  const float temperature = k.sp[0];
  const uint32_t transmit = (uint32_t)k.si[0];
  float rho[3], sab[3], ssc[3];
  for (int ch = 0; ch < 3; ++ch) { rho[ch] = k.sp[1 + 3 * ch]; sab[ch] = k.sp[2 + 3 * ch]; ssc[ch] = k.sp[3 + 3 * ch]; }
  V3 path;
  if (all_eq(ipos1(s), ipos2(s))) path = sub(ipos2(s), npos(n));
  else path = sub(ipos2(s), ipos1(s));
  float ki = RC_V2K * length(nvel(n));
  V3 normvel = normalize(nvel(n));
  float sigma_s = (ssc[0] + ssc[1] + ssc[2]) / (2.f * ki * ki);
  float sigma_a = (sab[0] + sab[1] + sab[2]) * 2200.f / length(nvel(n));
  float sigma_tot = sigma_a + sigma_s;
  float mu = (rho[0] + rho[1] + rho[2]) * sigma_tot * 100.f;
  float p_trans = rm_expf(-mu * length(path));
  if (o_rand(n, tid, c.kg) < p_trans) {
    n[P] *= p_trans;
    set_pos(n, add(ipos2(s), mul(0.0001f, normalize(path))));
    n[TOF] += s[7];
    if (transmit == 0) n[DIE] = 1.0f;
    n[SC] = (float)k.idx;
    *iidx = 0;
    reset_isect(s);
    return;
  } else {
    n[P] *= (1 - p_trans) * sigma_s / sigma_tot;
  }
  float eta = o_rand(n, tid, c.kg);
  float path_length = (-1.f / mu) * rm_logf(1 - eta * (1 - rm_expf(-mu * length(path))));
  float u = o_rand(n, tid, c.kg);
  u *= sigma_s;
  uint32_t flag = 0;
  float b1 = ssc[0] / (2.f * ki * ki), b2 = (ssc[0] + ssc[1]) / (2.f * ki * ki);
  if (u < b1) flag = 1;
  else if (u > b1 && u < b2) flag = 2;
  else if (u > b2) flag = 3;
  float omega = 0.0f, Q = 0.0f;
  if (flag >= 1 && flag <= 3) {
    int ch = (int)flag - 1;
    sample_distn(n, tid, c.kg, k.table[4 * ch], k.table[4 * ch + 1], k.table[4 * ch + 2],
                 k.table[4 * ch + 3], (uint32_t)k.si[1 + 2 * ch], (uint32_t)k.si[2 + 2 * ch],
                 &omega, &Q);
  }
  if (ki * ki < (RC_E2KS * omega)) {
    n[DIE] = 1;
    *iidx = 0;
    reset_isect(s);
    return;
  }
  float kf;
  if (o_rand(n, tid, c.kg) > 0.5f * rm_expf(-omega / (RC_KB * temperature))) {
    kf = sqrtf(ki * ki - RC_E2KS * omega);
    n[SE] = omega;
  } else {
    kf = sqrtf(ki * ki + RC_E2KS * omega);
    n[SE] = -omega;
  }
  float arg = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
  if (fabsf(arg) > 1) {
    n[DIE] = 1;
    *iidx = 0;
    reset_isect(s);
    return;
  }
  float theta = rm_acosf(arg);
  V3 oldvel = nvel(n);
  float z = -(n[3] + n[4]) / (n[5]);
  V3 perp = normalize(v3(1.f, 1.f, z));
  float alpha = 2 * RC_PI * o_rand(n, tid, c.kg);
  perp = rotate_about_axis(alpha, normvel, perp);
  normvel = rotate_about_axis(theta, perp, normvel);
  float TOFs = path_length / length(nvel(n));
  n[SD] = Q;
  if (all_eq(ipos1(s), ipos2(s))) {
    set_pos(n, mul(path_length, path));
    n[TOF] += TOFs;
  } else {
    set_pos(n, add(ipos1(s), mul(path_length, path)));
    n[TOF] += s[3] + TOFs;
  }
  set_vel(n, mulv(mulv(normvel, kf), RC_K2V));
  V3 q_norm = normalize(mulv(sub(oldvel, nvel(n)), RC_V2K));
  if (flag == 2) {
    set_pol(n, mulv(npol(n), -1.0f / 3.0f));
  } else if (flag == 3) {
    float dp = dot(npol(n), q_norm);
    set_pol(n, mulv(v3(-q_norm.x, -q_norm.y, -q_norm.z), dp));
  }
  n[SC] = (float)k.idx;
  *iidx = 0;
  reset_isect(s);
}

/* powderN — mcramp/scat/powderN.cl:5-156.  table[0] = sigma_scat*v^2 per
 * line, table[1] = q per line; sp[0] = sigma_abs*v, sp[1] = d_phi;
 * si[0] = num_lines, si[1] = transmit.  The cumulative walk stops at the
 * last line (the reference would read past the table), q_chosen starts at
 * 0, and a hard cap ends the retry loop when arg is never < 1 nor > 1. */
void s_powdern(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  uint32_t tid = c.tid_base + (uint32_t)i;
  const float* ssv2 = k.table[0];
  const float* qv = k.table[1];
  const float sigma_abs_v = k.sp[0], d_phi = k.sp[1];
  const uint32_t num_lines = (uint32_t)k.si[0];
  const uint32_t transmit = (uint32_t)k.si[1];
  V3 path;
  if (all_eq(ipos1(s), ipos2(s))) path = sub(ipos2(s), npos(n));
  else path = sub(ipos2(s), ipos1(s));
  float full_path_length = length(path);
  float vel = length(nvel(n));
  float sigma_abs = sigma_abs_v * 2200.0f / vel;
  float sum_sigma_scat = 0.0f, sigma_scat;
  for (uint32_t j = 0; j < num_lines; j++) {
    sigma_scat = ssv2[j] / (vel * vel * RC_V2K * RC_V2K);
    sum_sigma_scat += sigma_scat;
  }
  float p_inter = 1 - rm_expf(-(sum_sigma_scat + sigma_abs) * full_path_length);
  if (o_rand(n, tid, c.kg) > p_inter) {
    n[P] *= 1 - p_inter;
    set_pos(n, add(ipos2(s), mul(0.0001f, normalize(path))));
    n[TOF] += s[7];
    if (transmit == 0) n[DIE] = 1.0f;
    n[SC] = (float)k.idx;
    *iidx = 0;
    reset_isect(s);
    return;
  }
  uint32_t attempts = 0;
  float arg = 0.0f, q_chosen = 0.0f;
  while (true) {
    float u = o_rand(n, tid, c.kg);
    float v = 0.0f;
    uint32_t j = 0;
    while (v < u && j < num_lines) {
      sigma_scat = ssv2[j] / (vel * vel * RC_V2K * RC_V2K);
      q_chosen = qv[j];
      v += sigma_scat / sum_sigma_scat;
      j++;
    }
    arg = q_chosen * RC_K2V / (2.0f * vel);
    if (arg < 1.0f) break;
    else if ((arg > 1.0f && attempts > 2 * num_lines) || attempts > RC_POWDER_HARD_CAP) {
      if (!(arg > 1.0f && attempts > 2 * num_lines)) c.flags->fetch_or(RAMP_F_POWDER_CAP);
      n[DIE] = 1;
      *iidx = 0;
      reset_isect(s);
      return;
    }
    attempts++;
  }
  float twotheta = 2.0f * rm_asinf(arg);
  float pen_depth = -rm_logf(1.0f - o_rand(n, tid, c.kg) * (1.0f - p_inter)) / (sigma_abs + sum_sigma_scat);
  V3 beam_para = normalize(nvel(n));
  V3 beam_perp = cross(beam_para, v3(0.0f, 1.0f, 0.0f));
  if (length(beam_perp) < 1e-3f) beam_perp = normalize(cross(beam_para, v3(1.0f, 0.0f, 0.0f)));
  else beam_perp = normalize(beam_perp);
  float phi;
  if (d_phi != 0.0f) {
    phi = (2.0f * o_rand(n, tid, c.kg) - 1.0f) * (d_phi * RC_PI / 180.0f);
    if (o_rand(n, tid, c.kg) > 0.5f) phi += RC_PI;
    phi += RC_PI / 2.0f;
  } else {
    phi = 2.0f * RC_PI * o_rand(n, tid, c.kg);
  }
  beam_perp = rotate_about_axis(phi, beam_para, beam_perp);
  beam_para = rotate_about_axis(twotheta, beam_perp, beam_para);
  if (all_eq(ipos1(s), ipos2(s))) {
    set_pos(n, add(npos(n), mul(pen_depth, path)));
    n[TOF] += length(mul(pen_depth, path)) / length(nvel(n));
  } else {
    set_pos(n, add(ipos1(s), mul(pen_depth, path)));
    n[TOF] += s[7] - s[3];
  }
  set_vel(n, mul(vel, normalize(beam_para)));
  n[P] *= (1 - rm_expf(-(sum_sigma_scat + sigma_abs) * pen_depth)) * sum_sigma_scat /
          (sum_sigma_scat + sigma_abs);
  *iidx = 0;
  n[SC] = (float)k.idx;
  reset_isect(s);
}

/* detector — mcramp/scat/detector1D.cl:20-77.  sp[0..2] binning,
 * si[0] var, si[1] restore, si[2] n_bins; floor() can give index n_bins at
 * the top edge (a write past the buffer in the reference): dropped, counted */
void s_det1d(const Ctx& c, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const float min_var = k.sp[0], step_var = k.sp[1], max_var = k.sp[2];
  const uint32_t var = (uint32_t)k.si[0], restore = (uint32_t)k.si[1];
  const int64_t nb = k.si[2];
  float var_val = 0.0f;
  if (var == 0) { float L = length(nvel(n)); var_val = RC_VS2E * (L * L); }
  else if (var == 1) var_val = rm_degrees(rm_atan2f(s[4], s[6]));
  else if (var == 2) var_val = (1.0e6f) * (n[TOF] + s[7]);
  else if (var == 3) var_val = 2 * RC_PI / (RC_V2K * length(nvel(n)));
  if (min_var <= var_val && var_val <= max_var) {
    uint32_t idx = (uint32_t)floorf((var_val - min_var) / step_var);
    if ((int64_t)idx < nb && k.tally) {
      atomic_add_f(&k.tally[idx], n[P]);
      atomic_add_f(&k.tally_err[idx], n[P] * n[P]);
    } else if (n[P] != 0.0f) {
      c.oob->fetch_add(1);
    }
  }
  if (restore == 0) {
    set_pos(n, ipos2(s));
    n[TOF] += s[7];
    n[DIE] = 1.f;
  }
  *iidx = 0;
  n[SC] = (float)k.idx;
  reset_isect(s);
}

/* axis variable of detector2D.cl:48-145; axis 1 divX/divY use the
 * intersection y where axis 2 uses vz (detector2D.cl:93,96 vs 145,148) */
inline float det2d_val(uint32_t var, int axis, const float* n, const float* s) {
  float X2 = s[4], Y2 = s[5], Z2 = s[6];
  switch (var) {
    case 0: return X2;
    case 1: return Y2;
    case 2: return rm_degrees(rm_atan2f(X2, Z2));
    case 3: return rm_degrees(rm_atan2f(Y2, sqrtf(X2 * X2 + Z2 * Z2)));
    case 4: return rm_sign(Y2) * rm_degrees(rm_acosf(X2 / sqrtf(X2 * X2 + Y2 * Y2)));
    case 5: return (1.0e6f) * (n[TOF] + s[7]);
    case 6: return rm_degrees(rm_atan2f(n[3], axis == 1 ? Y2 : n[5]));
    case 7: return rm_degrees(rm_atan2f(n[4], axis == 1 ? Y2 : n[5]));
    case 8: return 2 * RC_PI / (RC_V2K * length(nvel(n)));
    case 9: { float L = length(nvel(n)); return RC_VS2E * (L * L); }
    case 10: return rm_sign(X2) * rm_degrees(rm_atan2f(sqrtf(X2 * X2 + Y2 * Y2), Z2));
    default: return 0.0f;
  }
}

/* find_idx — mcramp/scat/detector2D.cl:18-27 */
inline int find_idx(float val, float b0, float b1, float b2) {
  if (b0 <= val && val <= b2) return (int)roundf((val - b0) / b1);
  return -1;
}

/* detector — mcramp/scat/detector2D.cl:31-186.  sp[0..2], sp[3..5] axis
 * binnings; si[0], si[1] axis vars; si[2], si[3] n1, n2; si[4] restore.
 * round() maps the top half bin to index n: inside the buffer that bleeds
 * into the next row as in the reference, past its end it is dropped. */
void s_det2d(const Ctx& c, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  const uint32_t v1 = (uint32_t)k.si[0], v2 = (uint32_t)k.si[1];
  const int n2 = k.si[3];
  const uint32_t restore = (uint32_t)k.si[4];
  int a1 = find_idx(det2d_val(v1, 1, n, s), k.sp[0], k.sp[1], k.sp[2]);
  int a2 = find_idx(det2d_val(v2, 2, n, s), k.sp[3], k.sp[4], k.sp[5]);
  if (!((a1 == -1) || (a2 == -1))) {
    int64_t flat = (int64_t)a1 * n2 + a2;
    if (flat >= 0 && flat < k.tally_len && k.tally) {
      atomic_add_f(&k.tally[flat], n[P]);
      atomic_add_f(&k.tally_err[flat], n[P] * n[P]);
    } else if (n[P] != 0.0f) {
      c.oob->fetch_add(1);
    }
  }
  if (restore == 0) {
    set_pos(n, ipos2(s));
    n[TOF] += s[7];
    n[DIE] = 1.f;
  }
  *iidx = 0;
  n[SC] = (float)k.idx;
  reset_isect(s);
}

/* SAttenuate (no reference counterpart): Beer-Lambert weight over the
 * mesh chord sum kept in sd by g_mesh; moves the neutron to the exit point
 * of the earliest-exit record.  sp[0] = mu [1/m]. */
void s_attenuate(const Ctx&, int64_t, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  float chord_len = n[SD] * length(nvel(n));
  n[P] *= rm_expf(-k.sp[0] * chord_len);
  set_pos(n, ipos2(s));
  n[TOF] += s[7];
  finish(n, s, iidx, k);
}

/* randnorm — mcramp/scat/monochromator.cl:10-20 (Box-Muller, cosine) */
inline float o_randnorm(float* n, uint32_t tid, const Keying& kg) {
  float u1 = o_rand(n, tid, kg);
  float u2 = o_rand(n, tid, kg);
  return sqrtf(-2.0f * rm_logf(u1)) * rm_cosf(2.0f * RC_PI * u2);
}

/* GAUSS(x, 0, rms) — mcramp/scat/monochromator.cl:5-8 */
inline float o_gauss(float x, float rms) {
  float d = x - 0.0f;
  return rm_expf(-d * d / (2.0f * rms * rms)) / (sqrtf(2.0f * RC_PI) * rms);
}

/* monochromator — mcramp/scat/monochromator.cl:22-195.
 * sp: slab_width, slab_height, gap, mosaic_h, mosaic_v, r0, d_spacing,
 * radius_vertical, radius_horizontal; si: n_horizontal, n_vertical;
 * table[0], table[1]: Gauss-Legendre nodes and weights */
void s_mono(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  uint32_t tid = c.tid_base + (uint32_t)i;
  const float slab_width = k.sp[0], slab_height = k.sp[1], gap = k.sp[2];
  const float mosaic_h = k.sp[3], mosaic_v = k.sp[4], r0 = k.sp[5], d_spacing = k.sp[6];
  const float radius_vertical = k.sp[7], radius_horizontal = k.sp[8];
  const uint32_t n_h = (uint32_t)k.si[0], n_v = (uint32_t)k.si[1];
  const float* gx = k.table[0];
  const float* gw = k.table[1];
  const uint32_t glen = (uint32_t)k.table_len[0];
  set_pos(n, ipos2(s));
  n[TOF] += s[7];
  float mos_rms_y = RC_MIN2RAD * mosaic_h / sqrtf(8.0f * rm_logf(2.0f));
  float mos_rms_z = RC_MIN2RAD * mosaic_v / sqrtf(8.0f * rm_logf(2.0f));
  float mos_rms_max = mos_rms_y > mos_rms_z ? mos_rms_y : mos_rms_z;
  float Q = 2.0f * RC_PI / d_spacing;
  float zmax = (((float)n_h * (slab_width + gap)) - gap) / 2.0f;
  float zmin = -zmax;
  float ymax = (((float)n_v * (slab_height + gap)) - gap) / 2.0f;
  float ymin = -ymax;
  if (n[2] > zmin && n[2] < zmax && n[1] > ymin && n[1] < ymax) {
    float col = ceilf((n[2] - zmin) / (slab_width + gap));
    float row = ceilf((n[1] - ymin) / (slab_height + gap));
    float tilt_h = radius_horizontal > 0.0f
        ? rm_asinf((col - (float)(n_h + 1) / 2.0f) * (slab_width + gap) / radius_horizontal)
        : 0.0f;
    float tilt_v = radius_vertical > 0.0f
        ? -rm_asinf((row - (float)(n_v + 1) / 2.0f) * (slab_height + gap) / radius_vertical)
        : 0.0f;
    float center_z = zmin + (col - 0.5f) * (slab_width + gap) - gap / 2.0f;
    float center_y = ymin + (row - 0.5f) * (slab_height + gap) - gap / 2.0f;
    V3 slab_pos = v3(0.0f, center_y, center_z);
    float slab_rot[3] = {0.0f, tilt_h, tilt_v};
    set_vel(n, frame_derotate(nvel(n), slab_rot));
    set_pos(n, sub(npos(n), slab_pos));
    set_pos(n, frame_derotate(npos(n), slab_rot));
    if (fabsf(n[2]) <= slab_width / 2.0f && fabsf(n[1]) <= slab_height / 2.0f) {
      V3 ki = mul(RC_V2K, nvel(n));
      float ratio = -2.0f * ki.x / Q;
      float Q_order = floorf(ratio + 0.5f);
      if (Q_order == 0.0f) Q_order = ratio < 0.0f ? -1.0f : 1.0f;
      if (Q_order < 0.0f) Q_order = -Q_order;
      V3 ku = normalize(ki);
      if (Q_order > 2.0f * length(ki) / Q) Q_order -= 1.0f;
      float q0 = Q_order * Q;
      float q0x = ratio < 0.0f ? -q0 : q0;
      float theta = rm_asinf(q0 / (2.0f * length(ki)));
      float delta = rm_asinf(fabsf(ku.x)) - theta;
      float l12 = sqrtf(ki.y * ki.y + ki.z * ki.z);
      float p_reflect = fabsf(r0) *
          rm_expf(-ki.z * ki.z / (l12 * l12) * delta * delta / (2.0f * mos_rms_y * mos_rms_y)) *
          rm_expf(-ki.y * ki.y / (l12 * l12) * delta * delta / (2.0f * mos_rms_z * mos_rms_z));
      if (o_rand(n, tid, c.kg) <= p_reflect) {
        float cos_2theta = rm_cosf(2.0f * theta);
        float k_sin_2theta = length(ki) * rm_sinf(2.0f * theta);
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
          float cos_phi = rm_cosf(w), sin_phi = rm_sinf(w);
          q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
          q.y = q.y / mos_rms_z;
          q.z = q.z / mos_rms_y;
          if (q.z * q.z + q.y * q.y < (25.0f / (2.0f / 3.0f)) * (q.x * q.x)) break;
          mos_sample *= (2.0f / 3.0f);
        }
        for (uint32_t g = 0; g < glen; g++) {
          float phi = w * gx[g];
          float cos_phi = rm_cosf(phi), sin_phi = rm_sinf(phi);
          q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
          p_reflect = o_gauss(q.z / q.x, mos_rms_y) * o_gauss(q.y / q.x, mos_rms_z);
          total += gw[g] * p_reflect;
        }
        total *= w;
        float phi = mos_sample * o_randnorm(n, tid, c.kg);
        float cos_phi = rm_cosf(phi), sin_phi = rm_sinf(phi);
        q = add(add(c1, mul(cos_phi, a)), mul(sin_phi, b));
        p_reflect = o_gauss(q.z / q.x, mos_rms_y) * o_gauss(q.y / q.x, mos_rms_z);
        set_vel(n, mul(RC_K2V, add(ki, q)));
        p_reflect /= total * o_gauss(phi, mos_sample);
        if (p_reflect > 1.0f) p_reflect = 1.0f;
        n[P] *= p_reflect;
      }
    }
    set_pos(n, frame_rotate(npos(n), slab_rot));
    set_pos(n, add(npos(n), slab_pos));
    set_vel(n, frame_rotate(nvel(n), slab_rot));
  }
  finish(n, s, iidx, k);
}

/* powder1 — mcramp/scat/powder1.cl:5-100.  sp: sigma_scat*v^2,
 * sigma_abs*v, q, d_phi */
void s_powder1(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  uint32_t tid = c.tid_base + (uint32_t)i;
  const float sigma_scat_v2 = k.sp[0], sigma_abs_v = k.sp[1], q = k.sp[2], d_phi = k.sp[3];
  n[TOF] += s[3];
  V3 path = sub(ipos2(s), ipos1(s));
  float full_path_length = length(path);
  float vel = length(nvel(n));
  float sigma_scat = sigma_scat_v2 / (vel * vel * RC_V2K * RC_V2K);
  float sigma_abs = sigma_abs_v * 2200.0f / vel;
  float p_scat = sigma_scat / (sigma_abs + sigma_scat);
  float p_inter = 1 - rm_expf(-(sigma_scat + sigma_abs) * full_path_length);
  float arg = q * RC_K2V / (2.0f * vel);
  if (arg > 1.0f) {
    finish(n, s, iidx, k);
    return;
  }
  float twotheta = 2.0f * rm_asinf(arg);
  n[P] *= p_scat;
  float pen_depth = -rm_logf(1.0f - o_rand(n, tid, c.kg) * (1.0f - p_inter)) /
                    (sigma_abs + sigma_scat);
  V3 beam_para = normalize(nvel(n));
  V3 beam_perp = cross(beam_para, v3(0.0f, 1.0f, 0.0f));
  if (length(beam_perp) < 1e-3f) beam_perp = normalize(cross(beam_para, v3(1.0f, 0.0f, 0.0f)));
  else beam_perp = normalize(beam_perp);
  float phi;
  if (d_phi != 0.0f) {
    phi = (2.0f * o_rand(n, tid, c.kg) - 1.0f) * (d_phi * RC_PI / 180.0f);
    if (o_rand(n, tid, c.kg) > 0.5f) phi += RC_PI;
    phi += RC_PI / 2.0f;
  } else {
    phi = 2.0f * RC_PI * o_rand(n, tid, c.kg);
  }
  beam_perp = rotate_about_axis(phi, beam_para, beam_perp);
  beam_para = rotate_about_axis(twotheta, beam_perp, beam_para);
  set_pos(n, add(ipos1(s), mul(pen_depth, path)));
  set_vel(n, mul(vel, normalize(beam_para)));
  n[TOF] += s[7] - s[3];
  n[P] *= full_path_length * sigma_scat * rm_expf(-(sigma_scat + sigma_abs) * full_path_length);
  finish(n, s, iidx, k);
}

/* rescal — mcramp/scat/rescal.cl:5-76; the event goes to k.tally[8 i..],
 * ev.s345 (never written by the reference) as 0.  sp: target xyz, E0, dE,
 * focus_r */
void s_rescal(const Ctx& c, int64_t i, float* n, float* s, uint32_t* iidx, const RampComp& k) {
  uint32_t tid = c.tid_base + (uint32_t)i;
  V3 target = v3(k.sp[0], k.sp[1], k.sp[2]);
  const float E0 = k.sp[3], dE = k.sp[4], focus_r = k.sp[5];
  V3 path = sub(ipos2(s), ipos1(s));
  set_pos(n, add(ipos1(s), mul(o_rand(n, tid, c.kg), path)));
  V3 ki = mul(RC_V2K, nvel(n));
  float l2 = length(target) * length(target);
  float costhetamax = sqrtf(l2 / (focus_r * focus_r + l2));
  float theta = rm_acosf(1.0f - o_rand(n, tid, c.kg) * (1.0f - costhetamax));
  float phi = o_rand(n, tid, c.kg) * 2.0f * RC_PI;
  V3 target_perp;
  if (target.x == 0.0f && target.z == 0.0f) target_perp = v3(1.0f, 0.0f, 0.0f);
  else target_perp = v3(-target.z, 0.0f, target.x);
  V3 target_perp_perp = cross(target, target_perp);
  V3 target_final = target;
  target_final = rotate_about_axis(theta, target_perp_perp, target_final);
  target_final = rotate_about_axis(phi, target, target_final);
  target_final = normalize(target_final);
  float Ef = E0 + dE * (1.0f - 2.0f * o_rand(n, tid, c.kg));
  float vf = RC_SE2V * sqrtf(Ef);
  set_vel(n, mul(vf, target_final));
  V3 kf = mul(RC_V2K, nvel(n));
  float lk = length(mul(RC_K2V, ki));
  if (k.tally && 8 * i + 8 <= k.tally_len) {
    float* ev = k.tally + 8 * i;
    ev[0] = ki.x - kf.x; ev[1] = ki.y - kf.y; ev[2] = ki.z - kf.z;
    ev[3] = 0.0f; ev[4] = 0.0f; ev[5] = 0.0f;
    ev[6] = n[P];
    ev[7] = RC_VS2E * (lk * lk) - Ef;
  } else {
    c.oob->fetch_add(1);
  }
  finish(n, s, iidx, k);
}

void scatter(const Ctx& c, const RampComp& k) {
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < c.n; ++i) {
    float* n = c.neutrons + 16 * i;
    float* s = c.isect + 8 * i;
    uint32_t* ii = c.iidx + i;
    if (!(*ii == k.idx)) continue;
    if (n[DIE] > 0.f) continue;
    switch (k.scat) {
      case RAMP_S_ARM: s_arm(c, i, n, s, ii, k); break;
      case RAMP_S_GUIDE: s_guide(c, i, n, s, ii, k); break;
      case RAMP_S_CHOPPER: s_chopper(c, i, n, s, ii, k); break;
      case RAMP_S_ISOTROPIC: s_isotropic(c, i, n, s, ii, k); break;
      case RAMP_S_POWDERN: s_powdern(c, i, n, s, ii, k); break;
      case RAMP_S_DET1D: s_det1d(c, i, n, s, ii, k); break;
      case RAMP_S_DET2D: s_det2d(c, i, n, s, ii, k); break;
      case RAMP_S_COUNTER: s_counter(c, i, n, s, ii, k); break;
      case RAMP_S_BEAMSTOP: s_beamstop(c, i, n, s, ii, k); break;
      case RAMP_S_ATTENUATE: s_attenuate(c, i, n, s, ii, k); break;
      case RAMP_S_MONO: s_mono(c, i, n, s, ii, k); break;
      case RAMP_S_POWDER1: s_powder1(c, i, n, s, ii, k); break;
      case RAMP_S_RESCAL: s_rescal(c, i, n, s, ii, k); break;
      default: break;
    }
  }
}

}  // namespace

/* ========================================================================
 * Exported C functions (loaded by oracle/__init__.py through ctypes)
 * ====================================================================== */
extern "C" {

int oracle_version(void) { return RAMP_ABI_VERSION; }

/* One chunk of Instrument.execute (mcramp.py:442-455): gen_prg, then every
 * block with the reference sequencing.  Tallies are host pointers. */
int oracle_execute_chunk(const RampSource* src, const RampComp* comps, int n_comps,
                         const RampBlock* blocks, int n_blocks, float* neutrons,
                         float* isect, uint32_t* iidx, int64_t n, int32_t num_sim,
                         int32_t seed, const RampRng* rng, uint32_t variant,
                         uint32_t tid_base, int threads, uint32_t* flags_out,
                         uint64_t* oob_out) {
  if (!src || !neutrons || !isect || !iidx || n < 0) return RAMP_E_INVALID;
  if (threads > 0) omp_set_num_threads(threads);
  std::atomic<uint64_t> oob(0);
  std::atomic<uint32_t> flags(0);
  Ctx c;
  c.neutrons = neutrons; c.isect = isect; c.iidx = iidx; c.n = n;
  c.kg.mode = rng ? rng->mode : 0;
  c.kg.variant = variant;
  c.kg.run_seed = rng ? rng->run_seed : 0;
  c.tid_base = tid_base + (rng ? rng->tid_base : 0u);
  c.oob = &oob; c.flags = &flags;
  if (src->kind == RAMP_SRC_FLAT) gen_flat(c, *src, num_sim, seed);
  else if (src->kind == RAMP_SRC_CONT) gen_cont(c, *src, num_sim, seed);
  else if (src->kind == RAMP_SRC_ISIS) gen_isis(c, *src, num_sim, seed);
  else return RAMP_E_UNSUPPORTED;
  for (int b = 0; b < n_blocks; ++b) {
    const RampBlock& B = blocks[b];
    if (B.first < 0 || B.first + B.count > n_comps) return RAMP_E_INVALID;
    if (B.linear) {
      for (int j = B.first; j < B.first + B.count; ++j) {
        transform(c, comps[j]);
        intersect(c, comps[j]);
        terminate(c, comps[j]);
        scatter(c, comps[j]);
        untransform(c, comps[j]);
      }
    } else {
      for (int e = 0; e < B.multi; ++e) {
        for (int j = B.first; j < B.first + B.count; ++j) {
          transform(c, comps[j]);
          intersect(c, comps[j]);
          untransform(c, comps[j]);
        }
        for (int j = B.first; j < B.first + B.count; ++j) {
          transform(c, comps[j]);
          scatter(c, comps[j]);
          untransform(c, comps[j]);
        }
      }
    }
  }
  if (flags_out) *flags_out = flags.load();
  if (oob_out) *oob_out = oob.load();
  return RAMP_OK;
}

/* Threefry-4x32-20 word x for (counter word 0, tid), reference key/ctr. */
void oracle_threefry(const uint32_t* ctr0, const uint32_t* tid, uint32_t* out_x, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t key[4] = {tid[i], 0xdecafbadu, 0xfacebeadu, 0x12345678u};
    const uint32_t ctr[4] = {ctr0[i], 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
    uint32_t o[4];
    threefry4x32_20(ctr, key, o);
    out_x[i] = o[0];
  }
}

/* rand() on a record (rand.h): returns the draw, advances rec[11]. */
float oracle_rand(float* rec16, uint32_t tid, int mode, uint32_t variant, uint32_t run_seed) {
  Keying kg; kg.mode = mode; kg.variant = variant; kg.run_seed = run_seed;
  return o_rand(rec16, tid, kg);
}

float oracle_reflectivity(float q, float R0, float Qc, float alpha, float m, float W) {
  return reflectivity(q, R0, Qc, alpha, m, W);
}

/* elementwise rmath evaluation, same function numbering as the device
 * debug entry point ramp_debug_math */
void oracle_math(int fn, const float* a, const float* b, float* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    float x = a[i], y = b ? b[i] : 0.0f;
    switch (fn) {
      case 0: out[i] = rm_expf(x); break;
      case 1: out[i] = rm_logf(x); break;
      case 2: out[i] = rm_sinf(x); break;
      case 3: out[i] = rm_cosf(x); break;
      case 4: out[i] = rm_atan2f(x, y); break;
      case 5: out[i] = rm_asinf(x); break;
      case 6: out[i] = rm_acosf(x); break;
      case 7: out[i] = rm_tanhf(x); break;
      case 8: out[i] = rm_expm1f(x); break;
      case 9: out[i] = reflectivity(x, 0.99f, 0.0219f, 3.0f, 2.0f, 0.003f); break;
      default: out[i] = 0.0f; break;
    }
  }
}

}  // extern "C"
