/*
 * fused.cu — dispatch of the fused persistent kernel (fused_kernel.cuh)
 * over its register caps, keying modes and layouts; the instantiations live
 * in fused_{3,4}{r,n}{s,b}.cu.
 */
#include "fused_kernel.cuh"

#define EXT(MB, MODE)                                                                       \
  extern template cudaError_t launch_fk<MB, MODE, false>(const FusedArgs&, int, int,      \
                                                         cudaStream_t);                   \
  extern template cudaError_t launch_fk<MB, MODE, true>(const FusedArgs&, int, int,       \
                                                        cudaStream_t);                    \
  extern template int occ_mm<MB, MODE>(int);
EXT(3, 0)
EXT(3, 1)
EXT(4, 0)
EXT(4, 1)

static int g_fused_minb = 4;

/* register cap: 3 or 4 CTAs of 256 threads per SM (at 2 the kernel is
 * never faster on GB300) */
void fused_set_min_blocks(int minb) { g_fused_minb = minb >= 4 ? 4 : 3; }

template <int MB, int MODE>
static cudaError_t launch_m(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  return a.variants ? launch_fk<MB, MODE, true>(a, block, grid, s)
                    : launch_fk<MB, MODE, false>(a, block, grid, s);
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.n_tasks <= 0) return cudaSuccess;
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  if (a.split < 0 || (a.split > 0 && (a.split >= a.n_comps || !a.surv))) return cudaErrorInvalidValue;
  if (g_fused_minb == 4)
    return a.rng.mode == 0 ? launch_m<4, 0>(a, block, grid, s) : launch_m<4, 1>(a, block, grid, s);
  return a.rng.mode == 0 ? launch_m<3, 0>(a, block, grid, s) : launch_m<3, 1>(a, block, grid, s);
}

int fused_max_blocks_per_sm(int block, int n_comps) {
  (void)n_comps;
  return g_fused_minb == 4 ? occ_mm<4, 0>(block) : occ_mm<3, 0>(block);
}
