/*
 * pins.c — TEST INFRASTRUCTURE ONLY.  Compiles two of the reference's own
 * headers, unmodified and in place, into a host library so the oracle's
 * restatement can be checked against the reference itself:
 *   mcramp/include/rand.h   rand(): Threefry-4x32-20 keyed by
 *                           (tid, 0xdecafbad, 0xfacebead, 0x12345678),
 *                           counter word 0 = sb, u01 conversion (via the
 *                           vendored Random123 headers)
 *   mcramp/include/ref.h    reflectivity_func() (supermirror)
 * Built by oracle/build.py (build_ref_pins) with
 *   gcc -include shim.h -I<reference>/mcramp/include
 *       -ftrivial-auto-var-init=zero
 * (shim.h renames the reference's rand() to ref_rand()).
 * The last flag gives ref.h's uninitialised `beta` the value 0, the
 * reading the restatement takes.  Output: oracle/_ref/libref_pins.so.
 */
#include "rand.h"
#include "ref.h"

float ref_pin_rand(float* rec16, unsigned tid) {
  return ref_rand((float16*)rec16, tid);
}

float ref_pin_reflectivity(float q, float R0, float Qc, float alpha, float m, float W) {
  return reflectivity_func(q, R0, Qc, alpha, m, W);
}

void ref_pin_threefry(const uint32_t* ctr0, const uint32_t* tid, uint32_t* out_x, long n) {
  for (long i = 0; i < n; ++i) {
    threefry4x32_key_t k = {{tid[i], 0xdecafbad, 0xfacebead, 0x12345678}};
    threefry4x32_ctr_t c = {{ctr0[i], 0xf00dcafe, 0xdeadbeef, 0xbeeff00d}};
    threefry4x32_ctr_t r = threefry4x32(c, k);
    out_x[i] = r.v[0];
  }
}
