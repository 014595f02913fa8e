/*
 * plan.h — device-side descriptors shared by the plain, fused and ABI
 * translation units of libramp_cuda.so.
 */
#ifndef RAMP_PLAN_H
#define RAMP_PLAN_H

#include <stdint.h>
#include "../../include/ramp.h"

/* Per-component descriptor as the kernels read it: the RampComp slots plus
 * the frame rotation matrix, precomputed on the host with the same float
 * operations as mcramp/include/geom.h:21-53 evaluates per work-item, and
 * device copies of the tables. */
struct alignas(16) CompDev {
  int32_t geom, scat;
  uint32_t idx, restore;
  float pos[3];
  float R[9];                  /* r00 r01 r02 r10 r11 r12 r20 r21 r22     */
  int32_t rotated;             /* any Euler angle non-zero                */
  float gp[RAMP_NGP];
  float sp[RAMP_NSP];
  int32_t gi[RAMP_NGI];
  int32_t si[RAMP_NSI];
  const float* tab[RAMP_NTAB]; /* device tables                           */
  int64_t tab_len[RAMP_NTAB];
  float* tally;
  float* tally_err;
  int64_t tally_len;
  float aux[16];               /* per-kind constants derived on the host
                                  (guide: see guide_aux in abi.cu)         */
  int16_t dslot[6];            /* adjoint: gradient slot of each of this
                                  component's differentiable parameters
                                  (guide R0 Qc alpha m W; powder sigma_abs
                                  in slot 0), -1 when not differentiated  */
  int32_t adj_det;             /* adjoint: 1 for the loss detector        */
  const float* dLdH;           /* adjoint: dL/dH of the loss detector     */
  const float4* bvh_nodes;     /* mesh: 2 float4 per node                 */
  const float4* bvh_tris;      /* mesh: 3 float4 per triangle (v0,e1,e2)  */
  int32_t bvh_root_leaf;
  int32_t priv_off;            /* whole-chain launch with RampTune.privatize:
                                  offset (floats) of this detector's sum-p and
                                  sum-p^2 histograms in the CTA's shared
                                  memory; -1: the tallies go to global memory */
};

struct SrcDev {
  int32_t kind;
  int32_t pad;
  float p[16];
  float dmax[3];               /* maxwell(k_B T_i, T_i) (cont_mod.cl:25-27) */
  int32_t dslot_T;             /* adjoint: gradient slot of the common
                                  moderator temperature, -1 when not
                                  differentiated                          */
  const float* tab[4];         /* MISIS: flux CDF, time bins, energy edges,
                                  cumulative flux at the edges (device)   */
  int32_t n_t, n_e;            /* MISIS: time bins, energy edges          */
  float okt[3];                /* MCont: 1 / (k_B T_q), and okt^1.5 as      */
  float okc[3];                /* maxwell_energy_distn computes them       */
  uint32_t zero_terms;         /* MCont: bit q set when term q (1 or 2) is
                                  exactly +0 for every energy the source
                                  can draw (I_q = 0, finite positive T_q and
                                  normalisation, E_min, E_max >= 0)       */
  uint32_t pad_z;
};

struct RngDev {
  int32_t mode;
  uint32_t run_seed;
  uint32_t tid_base;
  uint32_t one;              /* 1, set by the host (Threefry's multiplier of
                                its adds, device.cuh: the launchers refuse
                                any other value) */
  const int32_t* seed_dev;   /* when set, the chunk seed is read here */
};

/* Device status block owned by a plan. */
struct StatusDev {
  unsigned int flags;
  unsigned int pad;
  unsigned long long oob;
  unsigned long long workq;    /* work-queue head of the persistent kernel */
  unsigned long long surv;     /* survivors appended by a split launch's stage A */
  unsigned long long workq_b;  /* work-queue head of its stage B */
  unsigned long long workq_c;  /* the mesh walk's finishing stage (PHASE 5) */
};

#define RAMP_MAX_COMPS 64
#define RAMP_MAX_DIFF 32   /* differentiable parameters per adjoint launch */

struct VariantDev {
  SrcDev src;
  int64_t n;
  int32_t num_sim;
  int32_t seed;
  const CompDev* comps;        /* n_comps descriptors in device memory    */
  int64_t item_off;            /* batched split: first survivor work item */
};

#endif /* RAMP_PLAN_H */
