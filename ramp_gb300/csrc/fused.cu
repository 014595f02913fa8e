/*
 * fused.cu — the fused path: one persistent kernel runs the whole chain
 * (moderator, every block and component) with each neutron in registers;
 * nothing but the tallies touches HBM.  Work is a list of tasks
 * (variant, first neutron, count); CTAs claim tasks from a device counter
 * and stage the claimed variant's component descriptors in shared memory,
 * so many instrument variants with uneven neutron counts share one launch.
 *
 * A neutron's history depends only on its index within its variant, the
 * variant's seed and the keying mode (counter-based RNG), so results are
 * independent of the task order and identical to the plain path.
 */
#include "device.cuh"
#include "launch.h"

#define FUSED_MAX_BLOCKS 32

__global__ void __launch_bounds__(256)
k_fused(const FusedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CompDev* sc = reinterpret_cast<CompDev*>(smem_raw);
  __shared__ RampBlock s_blocks[FUSED_MAX_BLOCKS];
  __shared__ SrcDev s_src;
  __shared__ long long s_task;
  __shared__ int s_var;
  __shared__ int64_t s_vn;
  __shared__ int32_t s_num_sim, s_seed;

  for (int b = threadIdx.x; b < a.n_blocks; b += blockDim.x) s_blocks[b] = a.blocks[b];
  if (threadIdx.x == 0) s_var = -1;
  __syncthreads();

  const int ncomp = a.n_comps;
  const int words = (int)(ncomp * sizeof(CompDev) / sizeof(int4));
  for (;;) {
    if (threadIdx.x == 0) s_task = (long long)atomicAdd(&a.st->workq, 1ull);
    __syncthreads();
    const long long t = s_task;
    if (t >= a.n_tasks) break;
    TaskDev T;
    if (a.tasks) {
      T = a.tasks[t];
    } else {
      T.variant = 0;
      T.start = t * a.task_size;
      int64_t rem = a.single.n - T.start;
      T.count = (int32_t)(rem < a.task_size ? rem : a.task_size);
    }
    if (T.variant != s_var) {
      __syncthreads();
      const VariantDev* V = a.variants ? a.variants + T.variant : &a.single;
      const int4* srcw = reinterpret_cast<const int4*>(V->comps);
      int4* dstw = reinterpret_cast<int4*>(sc);
      for (int w = threadIdx.x; w < words; w += blockDim.x) dstw[w] = srcw[w];
      if (threadIdx.x == 0) {
        s_src = V->src;
        s_vn = V->n;
        s_num_sim = V->num_sim;
        s_seed = V->seed;
        s_var = T.variant;
      }
      __syncthreads();
    }
    const int var = T.variant;
    for (int j = threadIdx.x; j < T.count; j += blockDim.x) {
      const int64_t i = T.start + j;
      Nt n;
      Rng r;
      rng_init(r, a.rng.mode, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed);
      const bool carry = (a.carry_sb != nullptr);
      float old_sb = carry ? a.carry_sb[i] : 0.0f;
      uint32_t ii = carry ? a.carry_iidx[i] : 0u;
      generate(s_src, n, old_sb, s_num_sim, s_seed, r);
      for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
        const RampBlock B = s_blocks[b];
        if (B.linear) {
          for (int k = B.first; k < B.first + B.count; ++k) {
            if (n.die > 0.f) break;
            comp_linear(sc[k], n, ii, r, a.st);
          }
        } else {
          block_nonlinear(sc, B.first, B.count, B.multi, n, ii, r, a.st);
        }
      }
      if (carry) {
        a.carry_sb[i] = n.sb;
        a.carry_iidx[i] = ii;
      }
    }
    __syncthreads();
  }
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.n_tasks <= 0) return cudaSuccess;
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  size_t smem = (size_t)a.n_comps * sizeof(CompDev);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(RAMP_MAX_COMPS * sizeof(CompDev)));
    attr_set = true;
  }
  k_fused<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

int fused_max_blocks_per_sm(int block, int n_comps) {
  int nb = 0;
  size_t smem = (size_t)n_comps * sizeof(CompDev);
  cudaFuncSetAttribute(k_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(RAMP_MAX_COMPS * sizeof(CompDev)));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused, block, smem) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}
