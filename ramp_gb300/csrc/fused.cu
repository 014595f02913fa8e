/*
 * fused.cu — dispatch of the fused persistent kernel (fused_kernel.cuh)
 * over its register caps, keying modes, layouts and kind sets, and the
 * sequencing of a split launch (stage A, then stage B).  The kernels are
 * instantiated one per translation unit (fused_inst.cu).
 */
#include "fused_kernel.cuh"

#define PH(MB, MODE, B, PHASE, X)                                                           \
  extern template cudaError_t launch_phase<MB, MODE, B, PHASE, X>(const FusedArgs&, int, int, \
                                                                  cudaStream_t);
#define ONE_MODE(MB, MODE)                                                                  \
  PH(MB, MODE, false, 0, false) PH(MB, MODE, false, 1, false) PH(MB, MODE, false, 2, false) \
  PH(MB, MODE, true, 0, false) PH(MB, MODE, true, 1, false) PH(MB, MODE, true, 2, false)    \
  PH(MB, MODE, false, 0, true) PH(MB, MODE, false, 1, true) PH(MB, MODE, false, 2, true)    \
  PH(MB, MODE, true, 0, true) PH(MB, MODE, false, 4, false) PH(MB, MODE, true, 4, false)    \
  extern template int occ_mm<MB, MODE>(int);
ONE_MODE(3, 0)
ONE_MODE(3, 1)
ONE_MODE(4, 0)
ONE_MODE(4, 1)

/* one register cap, keying mode, layout and kind set: the whole chain, or
 * stage A then stage B of a split launch (the batched one-launch layout
 * runs the extended kinds whole) */
template <int MB, int MODE, bool BATCHED, bool EXT>
static cudaError_t launch_fk(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if constexpr (!EXT) {
    if (a.walk) {
      const cudaError_t e = launch_phase<MB, MODE, BATCHED, 1, false>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 4, false>(a, block, grid, s);
    }
  }
  if constexpr (!(BATCHED && EXT)) {
    if (a.split > 0) {
      const cudaError_t e = launch_phase<MB, MODE, BATCHED, 1, EXT>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 2, EXT>(a, block, grid, s);
    }
  }
  return launch_phase<MB, MODE, BATCHED, 0, EXT>(a, block, grid, s);
}

template <int MB, int MODE>
static cudaError_t launch_m(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.ext)
    return a.variants ? launch_fk<MB, MODE, true, true>(a, block, grid, s)
                      : launch_fk<MB, MODE, false, true>(a, block, grid, s);
  return a.variants ? launch_fk<MB, MODE, true, false>(a, block, grid, s)
                    : launch_fk<MB, MODE, false, false>(a, block, grid, s);
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.variants ? a.n_variants <= 0 : a.n_tasks <= 0) return cudaSuccess;
  if (a.variants && a.n_variants > 65535) return cudaErrorInvalidValue;   /* grid rows */
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  if (a.split < 0 || (a.split > 0 && (a.split >= a.n_comps || !a.surv))) return cudaErrorInvalidValue;
  if (a.walk && (a.ext || a.split >= a.n_comps || !a.surv)) return cudaErrorInvalidValue;
  /* register cap: 3 or 4 CTAs of 256 threads per SM (at 2 the kernel is
     never faster on GB300) */
  if (a.minb != 3)
    return a.rng.mode == 0 ? launch_m<4, 0>(a, block, grid, s) : launch_m<4, 1>(a, block, grid, s);
  return a.rng.mode == 0 ? launch_m<3, 0>(a, block, grid, s) : launch_m<3, 1>(a, block, grid, s);
}

int fused_max_blocks_per_sm(int block, int minb) {
  return minb != 3 ? occ_mm<4, 0>(block) : occ_mm<3, 0>(block);
}
