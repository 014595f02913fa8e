/*
 * clshim.h — TEST INFRASTRUCTURE ONLY.  Lets the reference's own OpenCL C
 * kernels (mcramp/moderator/*.cl, geom/*.cl, scat/*.cl and the headers in
 * mcramp/include) compile as host C++ with g++, so that the oracle's
 * restatement can be checked against the reference's kernel code itself.
 *
 * It supplies what an OpenCL C compiler would: the address-space and
 * kernel qualifiers (empty here), the vector types float2/3/4/8/16 with
 * the component names (.s0-.sf, .x-.w) and the multi-component swizzles
 * the kernels use (.s012, .s345, ...), component-wise vector arithmetic,
 * vector comparisons returning integer masks with all(), and the built-in
 * functions the kernels call (geometric: dot, cross, length, normalize;
 * math: cos, sin, sqrt, exp, log, pow, acos, asin, atan2, tanh, fmod,
 * floor, ceil, round, fabs, sign, min, max, degrees; atomic_cmpxchg;
 * get_global_id, bound to the host loop index of the running work item).
 *
 * Math: with REFCL_RMATH the transcendental built-ins are the functions of
 * ramp_gb300/csrc/rmath.h (the library the oracle and the CUDA kernels
 * share), so that the oracle and the reference code can be compared bit
 * for bit and every difference is one of restatement; without it they are
 * the C library's single-precision functions, an independent
 * implementation compared within a relative tolerance.
 *
 * The build (oracle/refcl/build.py) compiles with -fsingle-precision-constant
 * (unsuffixed floating constants are float, as on an OpenCL device without
 * cl_khr_fp64), -ffp-contract=off and -ftrivial-auto-var-init=zero (a scalar
 * read before it is written reads 0).  Vector variables declared without a
 * value hold an "undefined" pattern instead, which a store to memory skips
 * (see refcl_undef below).  The only change made to the
 * reference sources is the mechanical rewrite of OpenCL vector literals
 * "(floatN)(...)" / "(floatN){...}" to "floatN(...)" / "floatN{...}", which
 * C++ would otherwise parse as a cast of a comma expression.
 */
#ifndef RAMP_REFCL_SHIM_H
#define RAMP_REFCL_SHIM_H

#include <stdint.h>
#include <string.h>
#include <stddef.h>
#include <limits.h>

#ifdef REFCL_RMATH
#include "../../ramp_gb300/csrc/rmath.h"
#endif

/* Random123 (vendored by the reference) is included once, here, in the
 * global namespace: each kernel file is compiled inside a namespace of its
 * own and its #include of the Random123 headers is then skipped by their
 * include guards. */
#include <Random123/threefry.h>
#include <Random123/u01fixedpt.h>
}   /* the vendored u01fixedpt.h opens extern "C" { under C++ and never
       closes it (its closing brace is missing); close it here */

#define __kernel
#define __global
#define __local
#define __constant const
#define __private
#define global        /* isis_mod.cl:20 spells one qualifier without underscores */

typedef unsigned int uint;
typedef unsigned long ulong;
typedef unsigned char uchar;
typedef unsigned short ushort;

/* ---- work-item index: set by the host loop of the driver -------------- */
extern thread_local uint refcl_gid;
static inline uint get_global_id(uint) { return refcl_gid; }

/* ---- vector types ------------------------------------------------------ */
/* The bit pattern of an uninitialised vector component.  The reference's
 * box.cl declares its intersection record without initialising it and, on
 * a miss, stores it back unchanged (box.cl:10,52): the store of an undefined
 * value, which LLVM-based OpenCL compilers remove, so the record in memory
 * keeps its previous contents.  Vector components carry this pattern until
 * they are assigned, and a vector store skips them. */
static inline float refcl_undef() {
  const uint32_t u = 0x7fa5a5a5u;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline bool refcl_is_undef(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u == 0x7fa5a5a5u;
}

/* a multi-component swizzle: a view of components I... of the enclosing
 * vector (all union members start at the vector's first component) */
template <int... I> struct swz;

struct int3m { int s0, s1, s2; };               /* mask of a float3 comparison */
static inline int all(int3m m) { return (m.s0 < 0) && (m.s1 < 0) && (m.s2 < 0); }

#define REFCL_FILL                                                         \
  template <class S, class... A> void fill_(int k, const S& a, const A&... rest) { \
    static_assert(std::is_arithmetic<S>::value, "vector literal part");    \
    v[k] = (float)a; fill_(k + 1, rest...);                                \
  }                                                                        \
  template <class... A> void fill_(int k, const float2& a, const A&... rest); \
  template <class... A> void fill_(int k, const float3& a, const A&... rest); \
  template <class... A> void fill_(int k, const float4& a, const A&... rest); \
  template <class... A> void fill_(int k, const float8& a, const A&... rest); \
  template <int... I, class... A>                                          \
  void fill_(int k, const swz<I...>& s, const A&... rest) {                \
    const int idx[] = {I...};                                              \
    for (int j = 0; j < (int)sizeof...(I); ++j) v[k + j] = s.base()[idx[j]]; \
    fill_(k + (int)sizeof...(I), rest...);                                 \
  }                                                                        \
  void fill_(int) {}

struct float2;
struct float3;
struct float4;
struct float8;
struct float16;

template <int N> struct vec_of;
template <> struct vec_of<2> { typedef float2 type; };
template <> struct vec_of<3> { typedef float3 type; };
template <> struct vec_of<4> { typedef float4 type; };
template <> struct vec_of<8> { typedef float8 type; };
template <> struct vec_of<16> { typedef float16 type; };

template <int... I> struct swz {
  static constexpr int N = sizeof...(I);
  typedef typename vec_of<N>::type V;
  /* a swizzle only exists inside its vector: never copied on its own */
  swz() = default;
  swz(const swz&) = delete;
  float* base() { return reinterpret_cast<float*>(this); }
  const float* base() const { return reinterpret_cast<const float*>(this); }
  operator V() const;
  swz& operator=(const V& x);
  swz& operator=(const swz& o) { return *this = V(o); }
  template <int... J> swz& operator=(const swz<J...>& o) { return *this = V(o); }
  swz& operator+=(const V& x);
  swz& operator-=(const V& x);
  swz& operator*=(float s);
};

#define REFCL_VEC_COMMON(T, N)                                             \
  /* an uninitialised vector: every component holds the "undefined"     \
     pattern (a signalling NaN that arithmetic never produces) */          \
  T() { for (int k = 0; k < N; ++k) v[k] = refcl_undef(); }               \
  T(const T& o) { memcpy(v, o.v, sizeof(v)); }                             \
  /* storing a vector: components still undefined leave the destination   \
     as it was, as an optimising OpenCL compiler drops the store of an     \
     undefined value */                                                    \
  T& operator=(const T& o) {                                               \
    for (int k = 0; k < N; ++k)                                            \
      if (!refcl_is_undef(o.v[k])) v[k] = o.v[k];                          \
    return *this;                                                          \
  }                                                                        \
  /* (T)(scalar): every component; (T)(a, b, ...): the parts in order */   \
  template <class A0, class... A,                                          \
            class = typename std::enable_if<                               \
                !std::is_same<typename std::decay<A0>::type, T>::value>::type> \
  explicit T(const A0& a0, const A&... rest) {                             \
    init_(std::integral_constant<bool, sizeof...(A) == 0 &&                \
                                 std::is_arithmetic<A0>::value>(), a0, rest...); \
  }                                                                        \
  template <class A0> void init_(std::true_type, const A0& a0) {           \
    for (int k = 0; k < N; ++k) v[k] = (float)a0;                          \
  }                                                                        \
  template <class... A> void init_(std::false_type, const A&... a) { fill_(0, a...); } \
  REFCL_FILL

#define REFCL_FILL_VEC(T)                                                  \
  template <class... A> void T::fill_(int k, const float2& a, const A&... rest) { \
    v[k] = a.v[0]; v[k + 1] = a.v[1]; fill_(k + 2, rest...);               \
  }                                                                        \
  template <class... A> void T::fill_(int k, const float3& a, const A&... rest) { \
    for (int j = 0; j < 3; ++j) v[k + j] = a.v[j];                         \
    fill_(k + 3, rest...);                                                 \
  }                                                                        \
  template <class... A> void T::fill_(int k, const float4& a, const A&... rest) { \
    for (int j = 0; j < 4; ++j) v[k + j] = a.v[j];                         \
    fill_(k + 4, rest...);                                                 \
  }                                                                        \
  template <class... A> void T::fill_(int k, const float8& a, const A&... rest) { \
    for (int j = 0; j < 8; ++j) v[k + j] = a.v[j];                         \
    fill_(k + 8, rest...);                                                 \
  }

#include <type_traits>

struct float2 {
  union {
    float v[2];
    struct { float s0, s1; };
    struct { float x, y; };
  };
  REFCL_VEC_COMMON(float2, 2)
};
struct float3 {
  union {
    float v[3];
    struct { float s0, s1, s2; };
    struct { float x, y, z; };
    swz<0, 1, 2> s012;
    swz<0, 1> s01;
    swz<1, 2> s12;
    swz<0, 2> s02;
  };
  REFCL_VEC_COMMON(float3, 3)
};
struct float4 {
  union {
    float v[4];
    struct { float s0, s1, s2, s3; };
    struct { float x, y, z, w; };
    swz<0, 1, 2> s012;
    swz<0, 1, 2> xyz;
  };
  REFCL_VEC_COMMON(float4, 4)
};
struct float8 {
  union {
    float v[8];
    struct { float s0, s1, s2, s3, s4, s5, s6, s7; };
    struct { float x, y, z, w; };
    swz<0, 1, 2> s012;
    swz<4, 5, 6> s456;
    swz<0, 1, 2, 3> s0123;
    swz<4, 5, 6, 7> s4567;
  };
  REFCL_VEC_COMMON(float8, 8)
};
struct float16 {
  union {
    float v[16];
    struct { float s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; };
    struct { float x, y, z, w; };
    swz<0, 1, 2> s012;
    swz<3, 4, 5> s345;
    swz<4, 5, 6> s456;
    swz<6, 7, 8> s678;
    swz<1, 2> s12;
    swz<3, 5> s35;
    swz<0, 2> s02;
    swz<0, 1, 2, 3> s0123;
    swz<4, 5, 6, 7> s4567;
  };
  REFCL_VEC_COMMON(float16, 16)
};

REFCL_FILL_VEC(float2)
REFCL_FILL_VEC(float3)
REFCL_FILL_VEC(float4)
REFCL_FILL_VEC(float8)
REFCL_FILL_VEC(float16)

template <int... I> swz<I...>::operator V() const {
  V r;
  const int idx[] = {I...};
  for (int k = 0; k < N; ++k) r.v[k] = base()[idx[k]];
  return r;
}
template <int... I> swz<I...>& swz<I...>::operator=(const V& x) {
  const int idx[] = {I...};
  float tmp[N];
  for (int k = 0; k < N; ++k) tmp[k] = x.v[k];
  for (int k = 0; k < N; ++k) base()[idx[k]] = tmp[k];
  return *this;
}
template <int... I> swz<I...>& swz<I...>::operator+=(const V& x) {
  return *this = V(*this) + x;
}
template <int... I> swz<I...>& swz<I...>::operator-=(const V& x) {
  return *this = V(*this) - x;
}
template <int... I> swz<I...>& swz<I...>::operator*=(float s) {
  return *this = V(*this) * s;
}

/* ---- component-wise arithmetic (non-template, so swizzles convert) ----- */
#define REFCL_VEC_OPS(T, N)                                                \
  static inline T operator+(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] + b.v[k]; return r; } \
  static inline T operator-(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] - b.v[k]; return r; } \
  static inline T operator*(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] * b.v[k]; return r; } \
  static inline T operator/(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] / b.v[k]; return r; } \
  static inline T operator*(const T& a, float s) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] * s; return r; } \
  static inline T operator*(float s, const T& a) { T r; for (int k = 0; k < N; ++k) r.v[k] = s * a.v[k]; return r; } \
  static inline T operator/(const T& a, float s) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] / s; return r; } \
  static inline T operator+(const T& a, float s) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] + s; return r; } \
  static inline T operator-(const T& a, float s) { T r; for (int k = 0; k < N; ++k) r.v[k] = a.v[k] - s; return r; } \
  static inline T operator-(const T& a) { T r; for (int k = 0; k < N; ++k) r.v[k] = -a.v[k]; return r; } \
  static inline T& operator+=(T& a, const T& b) { for (int k = 0; k < N; ++k) a.v[k] += b.v[k]; return a; } \
  static inline T& operator-=(T& a, const T& b) { for (int k = 0; k < N; ++k) a.v[k] -= b.v[k]; return a; } \
  static inline T& operator*=(T& a, float s) { for (int k = 0; k < N; ++k) a.v[k] *= s; return a; } \
  static inline T& operator/=(T& a, float s) { for (int k = 0; k < N; ++k) a.v[k] /= s; return a; }

REFCL_VEC_OPS(float2, 2)
REFCL_VEC_OPS(float3, 3)
REFCL_VEC_OPS(float4, 4)
REFCL_VEC_OPS(float8, 8)
REFCL_VEC_OPS(float16, 16)

static inline int3m operator==(const float3& a, const float3& b) {
  int3m m = {a.v[0] == b.v[0] ? -1 : 0, a.v[1] == b.v[1] ? -1 : 0, a.v[2] == b.v[2] ? -1 : 0};
  return m;
}

/* convert_float16 / convert_real16_t (consts.h maps real_t to float) */
static inline float16 convert_float16(const float16& a) { return a; }
static inline float8 convert_float8(const float8& a) { return a; }
static inline float3 convert_float3(const float3& a) { return a; }
static inline float convert_float(float a) { return a; }

/* int4 for rand.h's union with the Threefry counter (plain struct) */
struct int4 { int x, y, z, w; };

/* ---- scalar and geometric built-ins --------------------------------------
 * In namespace ocl; each kernel namespace takes them with the
 * using-declarations of REFCL_BUILTINS, which hide the C library's
 * overloads of the same names in the global namespace. */
namespace ocl {
#ifdef REFCL_RMATH
static inline float cos(float x) { return rm_cosf(x); }
static inline float sin(float x) { return rm_sinf(x); }
static inline float exp(float x) { return rm_expf(x); }
static inline float log(float x) { return rm_logf(x); }
static inline float acos(float x) { return rm_acosf(x); }
static inline float asin(float x) { return rm_asinf(x); }
static inline float atan2(float y, float x) { return rm_atan2f(y, x); }
static inline float tanh(float x) { return rm_tanhf(x); }
/* the kernels call pow(x, 2.0f) and pow(x, 1.5f) only */
static inline float pow(float x, float y) {
  if (y == 2.0f) return x * x;
  if (y == 1.5f) return x * __builtin_sqrtf(x);
  return rm_expf(y * rm_logf(x));
}
#else
static inline float cos(float x) { return __builtin_cosf(x); }
static inline float sin(float x) { return __builtin_sinf(x); }
static inline float exp(float x) { return __builtin_expf(x); }
static inline float log(float x) { return __builtin_logf(x); }
static inline float acos(float x) { return __builtin_acosf(x); }
static inline float asin(float x) { return __builtin_asinf(x); }
static inline float atan2(float y, float x) { return __builtin_atan2f(y, x); }
static inline float tanh(float x) { return __builtin_tanhf(x); }
static inline float pow(float x, float y) { return __builtin_powf(x, y); }
#endif
static inline float sqrt(float x) { return __builtin_sqrtf(x); }
static inline float fabs(float x) { return __builtin_fabsf(x); }
static inline float floor(float x) { return __builtin_floorf(x); }
static inline float ceil(float x) { return __builtin_ceilf(x); }
static inline float round(float x) { return __builtin_roundf(x); }
static inline float fmod(float x, float y) { return __builtin_fmodf(x, y); }
static inline float degrees(float x) { return x * 57.2957802f; }
static inline float radians(float x) { return x * 0.0174532924f; }
static inline float sign(float x) {
  if (x > 0.0f) return 1.0f;
  if (x < 0.0f) return -1.0f;
  if (x != x) return 0.0f;
  return x;   /* +0 or -0 */
}
/* OpenCL min/max of floats: y if y < x (resp. x < y), else x */
static inline float min(float x, float y) { return y < x ? y : x; }
static inline float max(float x, float y) { return x < y ? y : x; }
static inline int min(int x, int y) { return y < x ? y : x; }
static inline int max(int x, int y) { return x < y ? y : x; }
static inline uint min(uint x, uint y) { return y < x ? y : x; }
static inline uint max(uint x, uint y) { return x < y ? y : x; }

static inline float dot(const float3& a, const float3& b) {
  return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2];
}
static inline float dot(const float2& a, const float2& b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1]; }
static inline float3 cross(const float3& a, const float3& b) {
  return float3(a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
                a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
static inline float length(const float3& a) { return sqrt(dot(a, a)); }
static inline float length(const float2& a) { return sqrt(dot(a, a)); }
static inline float3 normalize(const float3& a) {
  const float d = dot(a, a);
  if (d == 0.0f) return a;
  return a * (1.0f / sqrt(d));
}
static inline float2 normalize(const float2& a) {
  const float d = dot(a, a);
  if (d == 0.0f) return a;
  return a * (1.0f / sqrt(d));
}
}  // namespace ocl

#define REFCL_BUILTINS                                                     \
  using ocl::cos; using ocl::sin; using ocl::exp; using ocl::log;           \
  using ocl::acos; using ocl::asin; using ocl::atan2; using ocl::tanh;      \
  using ocl::pow; using ocl::sqrt; using ocl::fabs; using ocl::floor;       \
  using ocl::ceil; using ocl::round; using ocl::fmod; using ocl::degrees;   \
  using ocl::radians; using ocl::sign; using ocl::min; using ocl::max;      \
  using ocl::dot; using ocl::cross; using ocl::length; using ocl::normalize;

/* ---- atomics ------------------------------------------------------------- */
static inline uint atomic_cmpxchg(volatile uint* p, uint cmp, uint val) {
  uint expected = cmp;
  __atomic_compare_exchange_n((uint*)p, &expected, val, false, __ATOMIC_SEQ_CST,
                              __ATOMIC_SEQ_CST);
  return expected;
}

#endif /* RAMP_REFCL_SHIM_H */
