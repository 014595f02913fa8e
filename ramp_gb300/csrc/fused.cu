/*
 * fused.cu — the fused path: one persistent kernel runs the whole chain
 * (moderator, every block and component) with each neutron in registers;
 * nothing but the tallies touches HBM.  Work is claimed per warp: lane 0
 * takes the next item (128 neutrons of one variant) from a device counter
 * and broadcasts it, so warps never wait on each other (no CTA barrier).
 * Many instrument variants with uneven neutron counts share one launch
 * through an explicit task list (variant, first neutron, count); component
 * descriptors are read through the read-only cache (every lane of a warp
 * reads the same address).  The kernel is instantiated per RNG keying mode
 * (fewer live registers) and per register cap (__launch_bounds__ minimum
 * CTAs per SM, chosen by the autotuner; 3 is the measured best on GB300).
 *
 * A neutron's history depends only on its index within its variant, the
 * variant's seed and the keying mode (counter-based RNG), so results are
 * independent of the claiming order and identical to the plain path.
 */
#include "device.cuh"
#include "launch.h"

#define FUSED_MAX_BLOCKS 32
#define FUSED_WARP_TASK 128   /* neutrons a warp claims at once */

template <int MINB, int MODE>
__global__ void __launch_bounds__(256, MINB)
k_fused(const FusedArgs a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(&a.st->workq, 1ull);
    t = __shfl_sync(0xffffffffu, t, 0);
    int var;
    int64_t start, count;
    const VariantDev* V;
    if (a.tasks) {
      const int64_t spt = (a.task_size + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK;
      const int64_t j = (int64_t)(t / (unsigned long long)spt);
      if (j >= a.n_tasks) break;
      const int64_t k = (int64_t)(t % (unsigned long long)spt);
      const TaskDev T = a.tasks[j];
      var = T.variant;
      start = T.start + k * FUSED_WARP_TASK;
      count = (int64_t)T.count - k * FUSED_WARP_TASK;
      if (count <= 0) continue;
      if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
      V = a.variants + var;
    } else {
      var = 0;
      start = (int64_t)t * FUSED_WARP_TASK;
      if (start >= a.single.n) break;
      count = a.single.n - start;
      if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
      V = &a.single;
    }
    const CompDev* __restrict__ comps = V->comps;
    const int32_t num_sim = V->num_sim;
    const int32_t seed = (a.rng.seed_dev && !a.tasks) ? *a.rng.seed_dev : V->seed;
    for (int j = lane; j < count; j += 32) {
      const int64_t i = start + j;
      Nt n;
      Rng r;
      rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed);
      const bool carry = (a.carry_sb != nullptr);
      float old_sb = carry ? a.carry_sb[i] : 0.0f;
      uint32_t ii = carry ? a.carry_iidx[i] : 0u;
      generate(V->src, n, old_sb, num_sim, seed, r);
      for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
        const RampBlock B = a.blocks[b];
        if (B.linear) {
          for (int k = B.first; k < B.first + B.count; ++k) {
            if (n.die > 0.f) break;
            comp_linear(comps[k], n, ii, r, a.st);
          }
        } else {
          block_nonlinear(comps, B.first, B.count, B.multi, n, ii, r, a.st);
        }
      }
      if (carry) { a.carry_sb[i] = n.sb; a.carry_iidx[i] = ii; }
    }
  }
}

static int g_fused_minb = 3;

void fused_set_min_blocks(int minb) { g_fused_minb = minb < 1 ? 1 : (minb > 4 ? 4 : minb); }

template <int MINB>
static cudaError_t launch_mb(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.rng.mode == 0) k_fused<MINB, 0><<<grid, block, 0, s>>>(a);
  else k_fused<MINB, 1><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.n_tasks <= 0) return cudaSuccess;
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  switch (g_fused_minb) {
    case 1: return launch_mb<1>(a, block, grid, s);
    case 2: return launch_mb<2>(a, block, grid, s);
    case 4: return launch_mb<4>(a, block, grid, s);
    default: return launch_mb<3>(a, block, grid, s);
  }
}

template <int MINB>
static int occ(int block) {
  static int cached = 0;
  if (cached > 0) return cached;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused<MINB, 0>, block, 0) !=
      cudaSuccess || nb <= 0)
    return 1;
  cached = nb;
  return nb;
}

int fused_max_blocks_per_sm(int block, int n_comps) {
  (void)n_comps;
  switch (g_fused_minb) {
    case 1: return occ<1>(block);
    case 2: return occ<2>(block);
    case 4: return occ<4>(block);
    default: return occ<3>(block);
  }
}
