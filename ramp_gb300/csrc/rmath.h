/*
 * rmath.h — a small portable single-precision math library, compiled
 * unchanged for the host (gcc, -ffp-contract=off) and for sm_103a (nvcc,
 * -fmad=false).  Every function uses only IEEE-754 operations that both
 * targets round identically (+, -, *, /, sqrt, rint, floor, fabs, fmod,
 * copysign), so a value computed here on the CPU and on the GPU is the same
 * bit pattern.  That is what lets the CPU restatement of the reference
 * kernels and the CUDA kernels agree neutron by neutron.
 *
 * The reference evaluates OpenCL built-ins (exp, log, sin, cos, acos, asin,
 * atan2, tanh, pow) whose last bits are left to each OpenCL implementation;
 * this library is one such implementation.  Methods (all textbook):
 *   exp    Cody-Waite reduction by ln2 (two-part constant), Taylor degree 7
 *   expm1  Taylor degree 8 for |x| < ln2/2, exp(x)-1 outside
 *   log    reduction to [sqrt(1/2), sqrt(2)), s = f/(2+f), atanh series
 *          log(1+f) = f - (f^2/2 - s (f^2/2 + R(s^2)))
 *   sin/cos  Cody-Waite reduction by pi/2 (three-part constant, |k|<4096;
 *          double-precision reduction beyond), Taylor degree 9 / 10
 *   atan   reduction to |u| <= tan(pi/8) via u = (t-1)/(t+1), Taylor
 *          degree 19; atan2/asin/acos built on it with C99 special cases
 *   tanh   expm1(2|x|) / (expm1(2|x|) + 2)
 * Polynomial coefficients are the Taylor coefficients rounded to float.
 * Accuracy against float64 references is checked in the test suite (a few
 * ulp); exactness between host and device is checked on the GPU.
 */
#ifndef RAMP_RMATH_H
#define RAMP_RMATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define RM_FN static __host__ __device__ __forceinline__
#else
#define RM_FN static inline
#endif

#define RM_INF (__builtin_huge_valf())

RM_FN uint32_t rm_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
RM_FN float rm_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* p * 2^k for k in [-252, 254]; each step multiplies by an exact power of
 * two, so only the last multiplication can round (subnormal results).     */
RM_FN float rm_scale2(float p, int k) {
  if (k > 127) { p *= 1.70141183e38f; k -= 127; }
  if (k < -126) { p *= 1.17549435e-38f; k += 126; }
  if (k < -126) { p *= 1.17549435e-38f; k += 126; }
  return p * rm_u2f((uint32_t)(k + 127) << 23);
}

#define RM_LN2_HI 0.693145751953125f    /* 16 significant bits */
#define RM_LN2_LO 1.42860677e-06f
#define RM_LOG2E  1.44269502f
#define RM_PIO2_1 1.5703125f            /* 12 significant bits */
#define RM_PIO2_2 4.83751297e-04f       /* 12 significant bits */
#define RM_PIO2_3 7.54979013e-08f
#define RM_2OPI   0.636619747f
#define RM_PI_HI  3.14159274f
#define RM_PI_LO  -8.74227766e-08f
#define RM_PIO2_HI 1.57079637f
#define RM_PIO2_LO -4.37113883e-08f
#define RM_PIO4_HI 0.785398185f
#define RM_PIO4_LO -2.18556941e-08f

RM_FN float rm_expf(float x) {
  if (x != x) return x;
  if (x > 88.7228394f) return RM_INF;
  if (x < -103.972076f) return 0.0f;
  float k = rintf(x * RM_LOG2E);
  float r = (x - k * RM_LN2_HI) - k * RM_LN2_LO;
  float p = 1.0f + r * (1.0f + r * (0.5f + r * (0.166666672f + r * (0.0416666679f
            + r * (0.00833333377f + r * (0.00138888892f + r * 0.000198412701f))))));
  return rm_scale2(p, (int)k);
}

RM_FN float rm_expm1f(float x) {
  float a = fabsf(x);
  if (a < 0.346573591f) {
    if (a < 1.0e-9f) return x;
    return x + x * x * (0.5f + x * (0.166666672f + x * (0.0416666679f
           + x * (0.00833333377f + x * (0.00138888892f + x * (0.000198412701f
           + x * 2.48015876e-05f))))));
  }
  return rm_expf(x) - 1.0f;
}

RM_FN float rm_logf(float x) {
  if (x != x) return x;
  if (x < 0.0f) return (x - x) / (x - x);      /* NaN */
  if (x == 0.0f) return -RM_INF;
  if (x == RM_INF) return x;
  uint32_t u = rm_f2u(x);
  int e = 0;
  if (u < 0x00800000u) { x *= 8388608.0f; u = rm_f2u(x); e = -23; }
  e += (int)(u >> 23) - 127;
  float m = rm_u2f((u & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421354f) { m *= 0.5f; e += 1; }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float R = z * (0.666666687f + z * (0.400000006f + z * (0.285714298f
            + z * (0.222222224f + z * 0.181818187f))));
  float hfsq = 0.5f * f * f;
  float logm = f - (hfsq - s * (hfsq + R));
  float fe = (float)e;
  return fe * RM_LN2_HI + (logm + fe * RM_LN2_LO);
}

RM_FN void rm_sincosf(float x, float* sp, float* cp) {
  if (!(fabsf(x) < RM_INF)) { *sp = x - x; *cp = x - x; return; }
  float k = rintf(x * RM_2OPI);
  float r;
  int q;
  if (fabsf(k) < 4096.0f) {
    r = ((x - k * RM_PIO2_1) - k * RM_PIO2_2) - k * RM_PIO2_3;
    q = (int)k & 3;
  } else {
    double kd = rint((double)x * 0.63661977236758134);
    r = (float)((double)x - kd * 1.5707963267948966);
    q = (int)(kd - 4.0 * floor(kd * 0.25));
  }
  float z = r * r;
  float s = r + r * (z * (-0.166666672f + z * (0.00833333377f
            + z * (-0.000198412701f + z * 2.75573188e-06f))));
  float c = (1.0f - 0.5f * z) + z * z * (0.0416666679f + z * (-0.00138888892f
            + z * (2.48015876e-05f + z * -2.75573188e-07f)));
  switch (q) {
    case 0: *sp = s; *cp = c; break;
    case 1: *sp = c; *cp = -s; break;
    case 2: *sp = -s; *cp = -c; break;
    default: *sp = -c; *cp = s; break;
  }
}

RM_FN float rm_sinf(float x) { float s, c; rm_sincosf(x, &s, &c); return s; }
RM_FN float rm_cosf(float x) { float s, c; rm_sincosf(x, &s, &c); return c; }

/* atan for t in [0, 1] */
RM_FN float rm_atan01(float t) {
  float u = t, hi = 0.0f, lo = 0.0f;
  if (t > 0.414213568f) { u = (t - 1.0f) / (t + 1.0f); hi = RM_PIO4_HI; lo = RM_PIO4_LO; }
  float z = u * u;
  float a = u + u * (z * (-0.333333343f + z * (0.200000003f + z * (-0.142857149f
            + z * (0.111111112f + z * (-0.0909090936f + z * (0.0769230798f
            + z * (-0.0666666701f + z * (0.0588235296f + z * -0.0526315793f)))))))));
  return hi + (a + lo);
}

RM_FN float rm_atan2f(float y, float x) {
  if (x != x || y != y) return x + y;
  float ax = fabsf(x), ay = fabsf(y);
  float r;
  if (ay == 0.0f) {
    r = (rm_f2u(x) >> 31) ? RM_PI_HI : 0.0f;          /* x<0 or x==-0 */
    return copysignf(r, y);
  }
  if (ax == 0.0f) return copysignf(RM_PIO2_HI, y);
  if (ax == RM_INF) {
    if (ay == RM_INF) r = (x > 0.0f) ? RM_PIO4_HI : 2.35619450f;
    else r = (x > 0.0f) ? 0.0f : RM_PI_HI;
    return copysignf(r, y);
  }
  if (ay == RM_INF) return copysignf(RM_PIO2_HI, y);
  if (ay <= ax) r = rm_atan01(ay / ax);
  else r = (RM_PIO2_HI - rm_atan01(ax / ay)) + RM_PIO2_LO;
  if (x < 0.0f) r = (RM_PI_HI - r) + RM_PI_LO;
  return copysignf(r, y);
}

RM_FN float rm_asinf(float x) {
  return rm_atan2f(x, sqrtf((1.0f - x) * (1.0f + x)));
}

RM_FN float rm_acosf(float x) {
  return rm_atan2f(sqrtf((1.0f - x) * (1.0f + x)), x);
}

RM_FN float rm_tanhf(float x) {
  float a = fabsf(x);
  if (a != a) return x;
  if (a > 9.0f) return copysignf(1.0f, x);
  if (a < 2.44140625e-4f) return x;
  float em = rm_expm1f(2.0f * a);
  return copysignf(em / (em + 2.0f), x);
}

/* OpenCL degrees(): radians * (180/pi) */
RM_FN float rm_degrees(float x) { return x * 57.2957802f; }

/* OpenCL sign(): 1, -1, or the signed zero; 0 for NaN */
RM_FN float rm_sign(float x) {
  if (x > 0.0f) return 1.0f;
  if (x < 0.0f) return -1.0f;
  if (x != x) return 0.0f;
  return x;
}

#endif /* RAMP_RMATH_H */
