/*
 * fused.cu — dispatch of the fused persistent kernel (fused_kernel.cuh)
 * over its register caps, keying modes, layouts and kind sets, and the
 * sequencing of a split launch (stage A, then stage B).  The kernels are
 * instantiated one per translation unit (fused_inst.cu).
 */
#include "fused_kernel.cuh"

#define PH(MB, MODE, B, PHASE, KS)                                                          \
  extern template cudaError_t launch_phase<MB, MODE, B, PHASE, KS>(const FusedArgs&, int, int, \
                                                                   cudaStream_t);
/* kind sets: 0 the core kinds, 1 everything (extended kinds: MISIS source,
   SMonochromator, SPowder1, and the mesh), 2 the core kinds and the mesh */
#define ONE_MODE(MB, MODE)                                                                  \
  PH(MB, MODE, false, 0, 0) PH(MB, MODE, false, 1, 0) PH(MB, MODE, false, 2, 0)             \
  PH(MB, MODE, true, 0, 0) PH(MB, MODE, true, 1, 0) PH(MB, MODE, true, 2, 0)                \
  PH(MB, MODE, false, 0, 1) PH(MB, MODE, false, 1, 1) PH(MB, MODE, false, 2, 1)             \
  PH(MB, MODE, true, 0, 1)                                                                  \
  PH(MB, MODE, false, 0, 2) PH(MB, MODE, false, 1, 2) PH(MB, MODE, false, 2, 2)             \
  PH(MB, MODE, true, 0, 2) PH(MB, MODE, true, 1, 2) PH(MB, MODE, true, 2, 2)                \
  PH(MB, MODE, false, 4, 2) PH(MB, MODE, true, 4, 2)                                        \
  PH(MB, MODE, false, 5, 2) PH(MB, MODE, true, 5, 2)                                        \
  PH(MB, MODE, false, 3, 0) PH(MB, MODE, true, 3, 0)                                        \
  extern template int occ_mm<MB, MODE>(int);
ONE_MODE(3, 0)
ONE_MODE(3, 1)
ONE_MODE(4, 0)
ONE_MODE(4, 1)

/* ---- before the lean stage A: the speed look-ahead -------------------
 * Every history's first draw (its energy, hence its speed) is made here
 * and the speed-only bound (speed_run_blocks) applied; the indices of the
 * histories that may pass are appended, one atomic per warp, to a list in
 * word 18 of the variant's survivor slots (free until a walk uses it), its
 * length in the variant's workq_c.  The lean stage A then traces only the
 * listed histories, each regenerated from its key (the same operations,
 * so the same neutron).  Without carry buffers only; with a source other
 * than flat or MCont every history is listed. */
template <int MODE, bool BATCHED>
__global__ void __launch_bounds__(256) k_speed_keep(const FusedArgs a) {
  const int var = BATCHED ? (int)blockIdx.y : a.var_key;
  const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
  const int64_t n = V->n;
  const int64_t item0 = BATCHED ? V->item_off : 0;
  if (BATCHED && item0 + (n + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK > a.surv_items) return;
  const SrcDev& src = V->src;
  const bool speed = (src.kind == RAMP_SRC_FLAT || src.kind == RAMP_SRC_CONT) &&
                     a.carry_sb == nullptr && a.cull > 0;
  uint32_t* const keep = a.surv + (size_t)18 * a.surv_cap + item0 * FUSED_WARP_TASK;
  unsigned long long* const kc = a.workq_c + (BATCHED ? var : 0);
  const int32_t seed = (a.rng.seed_dev && !BATCHED) ? *a.rng.seed_dev : V->seed;
  /* the run's per-chopper constants, once per CTA */
  __shared__ SpeedRun run;
  if (threadIdx.x == 0) {
    run.n = 0;
    if (speed) speed_run_prepare(V->comps, 0, a.cull, src.p[0], src.p[1], src.p[2], src.p[3],
                                 src.p[4], &run);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {                                   /* warp-uniform */
    const int64_t i = base + lane;
    bool kept = false;
    if (i < n) {
      kept = true;
      if (speed && run.n > 0) {
        /* generate's first draw and speed (flat_mod.cl, cont_mod.cl:36) */
        Rng r;
        rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed);
        Nt nn;
        nn.sb = (float)seed + 0.0f;
        const float E_val = src.p[5] + (src.p[6] - src.p[5]) * draw(nn, r);
        kept = !speed_run_blocks(run, RC_SE2V * sqrtf(E_val));
      }
    }
    const unsigned m = __ballot_sync(FULL_MASK, kept);
    if (m == 0u) continue;
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(kc, (unsigned long long)__popc(m));
    at = __shfl_sync(FULL_MASK, at, 0);
    if (kept) keep[at + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
  }
}

/* one register cap, keying mode, layout and kind set: the whole chain, or
 * stage A then stage B of a split launch (the batched one-launch layout
 * runs the extended kinds whole; the mesh walk runs with the mesh kind set;
 * a split before component 0 of a core-kind chain, which only the chopper
 * look-ahead makes, has a stage A of its own without the component code) */
template <int MB, int MODE, bool BATCHED, int KS>
static cudaError_t launch_fk(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if constexpr (KS == 2) {
    if (a.walk) {      /* stage A, the walk, then the rest of the chain */
      cudaError_t e = launch_phase<MB, MODE, BATCHED, 1, 2>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      e = launch_phase<MB, MODE, BATCHED, 4, 2>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 5, 2>(a, block, grid, s);
    }
  }
  if constexpr (!(BATCHED && KS == 1)) {
    if (a.split > 0 || a.cull > 0) {
      cudaError_t e;
      if (KS == 0 && a.split == 0) {   /* the moderator alone: the lean stage A */
        const dim3 g((unsigned)grid, BATCHED ? (unsigned)a.n_variants : 1u);
        k_speed_keep<MODE, BATCHED><<<g, 256, 0, s>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = launch_phase<MB, MODE, BATCHED, 3, 0>(a, block, grid, s);
      } else
        e = launch_phase<MB, MODE, BATCHED, 1, KS>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 2, KS>(a, block, grid, s);
    }
  }
  return launch_phase<MB, MODE, BATCHED, 0, KS>(a, block, grid, s);
}

template <int MB, int MODE>
static cudaError_t launch_m(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  switch (a.ext) {
    case 1:
      return a.variants ? launch_fk<MB, MODE, true, 1>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 1>(a, block, grid, s);
    case 2:
      return a.variants ? launch_fk<MB, MODE, true, 2>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 2>(a, block, grid, s);
    default:
      return a.variants ? launch_fk<MB, MODE, true, 0>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 0>(a, block, grid, s);
  }
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.variants ? a.n_variants <= 0 : a.n_tasks <= 0) return cudaSuccess;
  if (a.variants && a.n_variants > 65535) return cudaErrorInvalidValue;   /* grid rows */
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  if (a.split < 0 || ((a.split > 0 || a.cull > 0) && (a.split >= a.n_comps || !a.surv)))
    return cudaErrorInvalidValue;
  if (a.cull > 0 && (a.walk || a.split + a.cull > a.n_comps || (a.variants && a.ext == 1)))
    return cudaErrorInvalidValue;
  if (a.walk && (a.ext != 2 || a.split >= a.n_comps || !a.surv || !a.workq_c))
    return cudaErrorInvalidValue;
  /* register cap: 3 or 4 CTAs of 256 threads per SM (at 2 the kernel is
     never faster on GB300) */
  if (a.minb != 3)
    return a.rng.mode == 0 ? launch_m<4, 0>(a, block, grid, s) : launch_m<4, 1>(a, block, grid, s);
  return a.rng.mode == 0 ? launch_m<3, 0>(a, block, grid, s) : launch_m<3, 1>(a, block, grid, s);
}

int fused_max_blocks_per_sm(int block, int minb) {
  return minb != 3 ? occ_mm<4, 0>(block) : occ_mm<3, 0>(block);
}
