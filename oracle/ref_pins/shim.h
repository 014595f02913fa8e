/*
 * shim.h — TEST INFRASTRUCTURE ONLY.  Force-included (gcc -include) when
 * the reference's own mcramp/include/rand.h and ref.h are compiled as C on
 * the host.  It supplies the OpenCL C vector types those headers name, as
 * plain structs; no reference source is modified or copied.
 */
#ifndef RAMP_REF_SHIM_H
#define RAMP_REF_SHIM_H
#include <stdint.h>
#include <stdlib.h>
#include <math.h>
/* rand.h defines float rand(float16*, uint); keep libc's rand(void) apart */
#define rand ref_rand
typedef unsigned int uint;
typedef struct { float s0, s1; } float2;
typedef struct { float s0, s1, s2; } float3;
typedef struct { float s0, s1, s2, s3; } float4;
typedef struct { float s0, s1, s2, s3, s4, s5, s6, s7; } float8;
typedef struct { float s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; } float16;
typedef struct { int x, y, z, w; } int4;
#endif
