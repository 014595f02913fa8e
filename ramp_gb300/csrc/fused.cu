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
      if (KS == 0 && a.split == 0)     /* the moderator alone: the lean stage A */
        e = launch_phase<MB, MODE, BATCHED, 3, 0>(a, block, grid, s);
      else
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
