/*
 * fused_inst.cu — one instantiation of the fused kernel (fused_kernel.cuh).
 * The build compiles this file once per template argument set, each with
 * -DFK_MINB (register cap: minimum CTAs per SM), -DFK_MODE (RNG keying),
 * -DFK_BATCHED (one launch, a grid row per variant), -DFK_PHASE (0 whole
 * chain, 1 stage A, 2 stage B, 4 stage B walking a mesh per lane) and
 * -DFK_EXT (kind set: 0 core kinds, 1 everything, 2 core kinds and the
 * mesh), so that the kernels compile in parallel.
 */
#include "fused_kernel.cuh"

#if !defined(FK_MINB) || !defined(FK_MODE) || !defined(FK_BATCHED) || !defined(FK_PHASE) || \
    !defined(FK_EXT)
#error "fused_inst.cu is compiled with -DFK_MINB, -DFK_MODE, -DFK_BATCHED, -DFK_PHASE, -DFK_EXT"
#endif

template cudaError_t launch_phase<FK_MINB, FK_MODE, (FK_BATCHED != 0), FK_PHASE, FK_EXT>(
    const FusedArgs&, int, int, cudaStream_t);

#if FK_PHASE == 0 && FK_BATCHED == 0 && FK_EXT == 0
template int occ_mm<FK_MINB, FK_MODE>(int);
#endif
