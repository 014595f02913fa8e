/*
 * rconst.h — the physical constants of the neutron chain, as the float
 * values the reference compiles (mcramp/include/consts.h:1-37).  The
 * reference's own values are kept, including kB = 8.6173*10e-2 (0.86173,
 * ten times meV/K; consts.h:35-36) and E2KS = 1/2.072.  Shared by the CUDA
 * kernels and the CPU oracle so both see identical bits.
 */
#ifndef RAMP_RCONST_H
#define RAMP_RCONST_H

#define RC_K_B     1.38066e-23f          /* J/K                consts.h:4  */
#define RC_PI      3.14159265f           /* M_PI               consts.h:8  */
#define RC_V2K     1.58825361e-3f        /* m/s -> 1/AA        consts.h:12 */
#define RC_K2V     629.622368f           /* 1/AA -> m/s        consts.h:16 */
#define RC_VS2E    5.22703725e-6f        /* (m/s)^2 -> meV     consts.h:24 */
#define RC_SE2V    437.393377f           /* sqrt(meV) -> m/s   consts.h:28 */
#define RC_E2KS    (1.0f / 2.072f)       /*                    consts.h:32 */
#define RC_KB      (8.6173f * 10e-2f)    /* 0.86173            consts.h:36 */
#define RC_EV_J    1.6021765e-22f        /* meV -> J      cont_mod.cl:20   */
#define RC_MIN2RAD (RC_PI / (180.0f * 60.0f))  /* arc minute -> rad consts.h:20 */

/* intersection record reset value (doc/writing/buffers.rst:50-80) */
#define RC_T_RESET 100000.0f

/* hard caps on loops the reference leaves unbounded: a neutron that
 * reaches one is killed and a status flag is raised                      */
#define RC_GUIDE_HARD_CAP   100000
#define RC_POWDER_HARD_CAP  100000

#endif /* RAMP_RCONST_H */
