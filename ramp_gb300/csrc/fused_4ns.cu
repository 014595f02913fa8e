/* fused kernel instantiations: register cap 4 CTAs per SM, native keying,
 * one instrument (one translation unit each, so they compile in parallel) */
#include "fused_kernel.cuh"

template cudaError_t launch_fk<4, 1, false>(const FusedArgs&, int, int, cudaStream_t);
template int occ_mm<4, 1>(int);
