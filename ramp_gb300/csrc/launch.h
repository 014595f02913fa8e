/*
 * launch.h — kernel launchers shared between the translation units of
 * libramp_cuda.so (host side).
 */
#ifndef RAMP_LAUNCH_H
#define RAMP_LAUNCH_H

#include <cuda_runtime.h>
#include "plan.h"

struct PlainArgs {
  float* soa;
  uint32_t* iidx;
  int64_t stride;
  int64_t n;
  RngDev rng;
  StatusDev* st;
};

cudaError_t launch_host_half(const CompDev& c, const PlainArgs& a, int leave, cudaStream_t s);
cudaError_t launch_gather_alive(const PlainArgs& a, uint32_t lanes, float* out, int64_t* scratch,
                                int64_t* total, cudaStream_t s);
cudaError_t launch_generate(const SrcDev& src, const PlainArgs& a, int32_t num_sim,
                            int32_t seed, cudaStream_t s);
cudaError_t launch_linear_comp(const CompDev& c, const PlainArgs& a, cudaStream_t s);
cudaError_t launch_nonlinear_block(const CompDev* comps_dev, int first, int count, int multi,
                                   bool mesh, const PlainArgs& a, cudaStream_t s);

struct FusedArgs {
  const VariantDev* variants;   /* device, n_variants entries (one grid row
                                   each); NULL: one variant, "single"      */
  int64_t n_tasks;              /* single: spans of task_size (caps the grid) */
  int64_t task_size;
  VariantDev single;
  const RampBlock* blocks;      /* device */
  int32_t n_blocks;
  int32_t n_comps;
  RngDev rng;
  float* carry_sb;              /* optional, single variant */
  uint32_t* carry_iidx;
  StatusDev* st;
  int32_t split;                /* survivor compaction before this component; 0: off */
  int32_t n_variants;           /* rows of a batched grid */
  uint32_t* surv;               /* split: SURV_WORDS x surv_cap survivor records */
  int64_t surv_cap;             /* slots: 128 per work item */
  uint32_t* surv_cnt;           /* survivors per work item */
  int64_t surv_items;
  unsigned long long* workq;    /* work-queue counter of this launch (batched:
                                   one per variant) */
  unsigned long long* workq_b;  /* stage-B work-queue counter(s) (split) */
  unsigned long long* workq_c;  /* the walk's finishing stage: work-queue
                                   counter(s) of PHASE 5 */
  int32_t var_key;              /* single variant: its index in the RNG key */
  int32_t minb;                 /* register cap: the build for 3 or 4 CTAs per SM */
  int32_t walk;                 /* split before the GMesh component `split` (may
                                   be 0): stage B walks the mesh per lane (PHASE 4) */
  int32_t ext;                  /* kind set of the kernels to run: 0 the core
                                   kinds; 1 the chain uses an extended kind
                                   (MISIS source, SMonochromator, SPowder1):
                                   everything (split only when not BATCHED);
                                   2 core kinds and GMesh / SAttenuate */
  int32_t priv_floats;          /* whole chain, one instrument: shared-memory
                                   floats of the private tallies (descriptors
                                   with priv_off >= 0); 0: off */
  int32_t cull;                 /* split launch: components of the chopper run
                                   at `split` (lookahead.h); stage A retires
                                   the neutrons that cannot pass it (without
                                   carry buffers).  0: off */
};
#define RAMP_PRIV_FLOATS 12288  /* shared memory for private tallies: 48 KB per CTA */
#define SURV_WORDS 18           /* 15 record lanes (die is 0), iidx, index, variant */
#define SURV_WORDS_WALK 24      /* and, after a mesh walk, its result: t of the
                                   two records, the chord (a double, two words),
                                   the crossing count and how the walk ended */

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s);
int fused_max_blocks_per_sm(int block, int minb);

struct AdjointArgs {
  SrcDev src;
  const CompDev* comps;         /* device, with the adjoint fields set     */
  const RampBlock* blocks;      /* device */
  int32_t n_blocks;
  int32_t nslot;
  int64_t n;
  int32_t num_sim;
  int32_t seed;
  RngDev rng;
  double* grad;
  int32_t lr;
  StatusDev* st;
  uint32_t* list;               /* pass 1 output: indices the loss detector counts */
  unsigned long long* list_count;
  int64_t list_cap;
  int32_t cull;                 /* pass 1: components of the chopper run at
                                   component 0 (lookahead.h), 0: none */
  uint32_t* keep;               /* with cull: the indices the look-ahead keeps */
  unsigned long long* keep_count;
};

cudaError_t launch_adjoint(const AdjointArgs& a, int grid, int passes, cudaStream_t s);

cudaError_t launch_seed_advance(int32_t* seed_dev, cudaStream_t s);
cudaError_t launch_debug_threefry(const uint32_t* c0, const uint32_t* tid, uint32_t* out,
                                  int64_t n, cudaStream_t s);
cudaError_t launch_debug_rng_peak(int64_t n, int32_t iters, uint32_t* out, cudaStream_t s);
cudaError_t launch_debug_l2_peak(const float4* buf, int64_t len4, int64_t n, int32_t iters,
                                 float* out, cudaStream_t s);
cudaError_t launch_debug_atomic_peak(float* bins, int64_t n_bins, int64_t n, int32_t iters,
                                     cudaStream_t s);
cudaError_t launch_debug_math(int fn, const float* a, const float* b, float* out, int64_t n,
                              cudaStream_t s);

#endif
