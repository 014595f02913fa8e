/*
 * fused_kernel.cuh — the fused path: one persistent kernel runs the whole chain
 * (moderator, every block and component) with each neutron in registers;
 * nothing but the tallies touches HBM.  Work is claimed per warp: lane 0
 * takes the next item (128 neutrons of one variant) from a device counter
 * and broadcasts it, so warps never wait on each other (no CTA barrier).
 * Many instrument variants with uneven neutron counts share one launch
 * through an explicit task list (variant, first neutron, count); component
 * descriptors are read through the read-only cache (every lane of a warp
 * reads the same address).  The kernel is instantiated per RNG keying mode
 * (fewer live registers) and per register cap (__launch_bounds__ minimum
 * CTAs per SM, chosen by the autotuner).
 *
 * A neutron's history depends only on its index within its variant, the
 * variant's seed and the keying mode (counter-based RNG), so results are
 * independent of the claiming order and identical to the plain path.
 * With a split point K the chain runs as two kernels: stage A (moderator
 * and components [0, K)) appends the neutrons still alive to a survivor
 * buffer in HBM, and stage B traces them through components [K, end) in
 * full warps (see fused_tail below).
 */
#ifndef RAMP_FUSED_KERNEL_CUH
#define RAMP_FUSED_KERNEL_CUH
#include "device.cuh"
#include "launch.h"

#define FUSED_MAX_BLOCKS 32
#define FUSED_WARP_TASK 128   /* neutrons a warp claims at once */
#define FULL_MASK 0xffffffffu

/* Without a carry buffer nothing but the tallies is observable, and every
 * later weight factor multiplies p while every tally adds p or p^2: a
 * neutron whose weight is exactly zero can only add zeros, so it is
 * retired at once (zx; the plain path, whose records are output, keeps
 * tracing it as the reference does). */

/*
 * PHASE 0: the whole chain per neutron.  PHASE 1: stage A of a split
 * launch — the moderator and components [0, split); the survivors of work
 * item t are stored at slots [128 t, 128 t + cnt[t]) of the survivor
 * buffer (no atomics) and finish in PHASE 2.  The bounds of both loops are kernel parameters, so the loop
 * counters and descriptor addresses stay warp-uniform.
 */
template <int MINB, int MODE, bool BATCHED, int PHASE, bool EXT>
__global__ void __launch_bounds__(256, MINB)
k_fused(const FusedArgs a);

/* PHASE 2: the survivors of stage A through components [split, end).
 * Stage A leaves the survivors of work item t at slots [128 t, 128 t +
 * cnt[t]); a warp claims SURV_GROUP items at a time and deals their
 * survivors out 32 to a pass.  A survivor is keyed by its own index and
 * variant, so it continues exactly where stage A left it. */
#define SURV_GROUP 8
template <int MODE, bool BATCHED, bool EXT>
DI void fused_tail(const FusedArgs& a) {
  const int lane = threadIdx.x & 31;
  const bool carry = (a.carry_sb != nullptr);
  const bool zx = !carry;
  const int K = a.split;
  const int64_t cap = a.surv_cap;
  for (;;) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(a.workq_b, 1ull);
    g = __shfl_sync(FULL_MASK, g, 0);
    const int64_t t0 = (int64_t)g * SURV_GROUP;
    if (t0 >= a.surv_items) break;
    const int c = (lane < SURV_GROUP && t0 + lane < a.surv_items) ? (int)a.surv_cnt[t0 + lane] : 0;
    int incl = c;
    for (int d = 1; d < SURV_GROUP; d <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, incl, d);
      if (lane >= d) incl += y;
    }
    const int excl = incl - c;
    const int total = __shfl_sync(FULL_MASK, incl, SURV_GROUP - 1);
    for (int q0 = 0; q0 < total; q0 += 32) {
      const int q = q0 + lane;
      int item = 0, base = 0;
      for (int k = 0; k < SURV_GROUP; ++k) {   /* last item starting at or before q */
        const int ek = __shfl_sync(FULL_MASK, excl, k);
        const int ck = __shfl_sync(FULL_MASK, c, k);
        if (ck > 0 && ek <= q) { item = k; base = ek; }
      }
      if (q >= total) continue;
      const int64_t s = (t0 + item) * FUSED_WARP_TASK + (q - base);
      const uint32_t* w = a.surv + s;
      Nt n;
      n.x = __uint_as_float(w[0 * cap]);   n.y = __uint_as_float(w[1 * cap]);
      n.z = __uint_as_float(w[2 * cap]);   n.vx = __uint_as_float(w[3 * cap]);
      n.vy = __uint_as_float(w[4 * cap]);  n.vz = __uint_as_float(w[5 * cap]);
      n.px = __uint_as_float(w[6 * cap]);  n.py = __uint_as_float(w[7 * cap]);
      n.pz = __uint_as_float(w[8 * cap]);  n.p = __uint_as_float(w[9 * cap]);
      n.t = __uint_as_float(w[10 * cap]);  n.sb = __uint_as_float(w[11 * cap]);
      n.sc = __uint_as_float(w[12 * cap]); n.sd = __uint_as_float(w[13 * cap]);
      n.se = __uint_as_float(w[14 * cap]);
      n.die = 0.0f;
      n.wr = 0u;
      uint32_t ii = w[15 * cap];
      const uint32_t idx = w[16 * cap], var = w[17 * cap];
      Rng r;
      rng_init(r, MODE, a.rng.tid_base + idx, var, a.rng.run_seed);
      const CompDev* __restrict__ comps = BATCHED ? a.variants[var].comps : a.single.comps;
      for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
        const RampBlock B = a.blocks[b];
        const int e = B.first + B.count;
        if (e <= K) continue;
        if (B.linear) {
          for (int k = B.first > K ? B.first : K; k < e; ++k) {
            if (n.die > 0.f) break;
            comp_linear<TallyOnly, EXT>(comps[k], n, ii, r, a.st, (TallyOnly*)nullptr, zx);
          }
        } else {
          block_nonlinear<TallyOnly>(comps, B.first, B.count, B.multi, n, ii, r, a.st);
        }
      }
      if (carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
    }
  }
}

template <int MINB, int MODE, bool BATCHED, int PHASE, bool EXT>
__global__ void __launch_bounds__(256, MINB)
k_fused(const FusedArgs a) {
  if constexpr (PHASE == 2) {
    fused_tail<MODE, BATCHED, EXT>(a);
    return;
  } else {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int KE = PHASE == 1 ? a.split : a.n_comps;
    for (;;) {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(a.workq, 1ull);
      t = __shfl_sync(FULL_MASK, t, 0);
      int var;
      int64_t start, count;
      const VariantDev* V;
      if (BATCHED) {
        const int64_t spt = (a.task_size + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK;
        const int64_t jt = (int64_t)(t / (unsigned long long)spt);
        if (jt >= a.n_tasks) break;
        const int64_t k = (int64_t)(t % (unsigned long long)spt);
        const TaskDev T = a.tasks[jt];
        var = T.variant;
        start = T.start + k * FUSED_WARP_TASK;
        count = (int64_t)T.count - k * FUSED_WARP_TASK;
        if (count <= 0) continue;
        if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
        V = a.variants + var;
      } else {
        var = a.var_key;
        start = (int64_t)t * FUSED_WARP_TASK;
        if (start >= a.single.n) break;
        count = a.single.n - start;
        if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
        V = &a.single;
      }
      const CompDev* __restrict__ comps = V->comps;
      const int32_t num_sim = V->num_sim;
      const int32_t seed = (a.rng.seed_dev && !BATCHED) ? *a.rng.seed_dev : V->seed;
      const bool carry = (a.carry_sb != nullptr);
      const bool zx = !carry;
      int kept = 0;      /* PHASE 1: survivors of this item so far (warp-uniform) */
      /* PHASE 1 keeps the whole warp in the loop for the ballot */
      const int jend = PHASE == 1 ? (int)((count + 31) & ~31ll) : (int)count;
      for (int j = lane; j < jend; j += 32) {
        const bool live = j < count;
        const int64_t i = start + j;
        Nt n;
        Rng r;
        uint32_t ii = 0u;
        if (live) {
          rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed);
          const float old_sb = carry ? a.carry_sb[i] : 0.0f;
          ii = carry ? a.carry_iidx[i] : 0u;
          generate<TallyOnly, EXT>(V->src, n, old_sb, num_sim, seed, r);
          if (zx && n.p == 0.0f) n.die = 1.0f;
          for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
            const RampBlock B = a.blocks[b];
            if (PHASE == 1 && B.first >= KE) break;
            if (B.linear) {
              const int e = (PHASE == 1 && B.first + B.count > KE) ? KE : B.first + B.count;
              for (int k = B.first; k < e; ++k) {
                if (n.die > 0.f) break;
                comp_linear<TallyOnly, EXT>(comps[k], n, ii, r, a.st, (TallyOnly*)nullptr, zx);
              }
            } else {
              block_nonlinear<TallyOnly>(comps, B.first, B.count, B.multi, n, ii, r, a.st);
            }
          }
        }
        if (PHASE == 0) {
          if (carry) { a.carry_sb[i] = n.sb; a.carry_iidx[i] = ii; }
          continue;
        }
        const bool alive = live && !(n.die > 0.f);
        if (live && !alive && carry) { a.carry_sb[i] = n.sb; a.carry_iidx[i] = ii; }
        const unsigned m = __ballot_sync(FULL_MASK, alive);
        const int rank = kept + __popc(m & lt);
        kept += __popc(m);
        if (!alive) continue;
        const int64_t s = (int64_t)t * FUSED_WARP_TASK + rank;   /* rank < 128 */
        if (s >= a.surv_cap) {          /* cannot happen: one slot per neutron of the item */
          raise_flag(a.st, RAMP_F_WORKQ);
          continue;
        }
        const int64_t cap = a.surv_cap;
        uint32_t* w = a.surv + s;
        w[0 * cap] = __float_as_uint(n.x);   w[1 * cap] = __float_as_uint(n.y);
        w[2 * cap] = __float_as_uint(n.z);   w[3 * cap] = __float_as_uint(n.vx);
        w[4 * cap] = __float_as_uint(n.vy);  w[5 * cap] = __float_as_uint(n.vz);
        w[6 * cap] = __float_as_uint(n.px);  w[7 * cap] = __float_as_uint(n.py);
        w[8 * cap] = __float_as_uint(n.pz);  w[9 * cap] = __float_as_uint(n.p);
        w[10 * cap] = __float_as_uint(n.t);  w[11 * cap] = __float_as_uint(n.sb);
        w[12 * cap] = __float_as_uint(n.sc); w[13 * cap] = __float_as_uint(n.sd);
        w[14 * cap] = __float_as_uint(n.se);
        w[15 * cap] = ii; w[16 * cap] = (uint32_t)i; w[17 * cap] = (uint32_t)var;
      }
      if (PHASE == 1 && lane == 0 && (int64_t)t < a.surv_items) a.surv_cnt[t] = (uint32_t)kept;
    }
  }
}

/* one launch of one instantiation; each is compiled in a translation unit
 * of its own (fused_inst.cu, built once per template argument set) and the
 * sequencing of phases lives in fused.cu */
template <int MINB, int MODE, bool BATCHED, int PHASE, bool EXT>
cudaError_t launch_phase(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  k_fused<MINB, MODE, BATCHED, PHASE, EXT><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

/* occupancy of the whole-chain kernel at this register cap (CTAs per SM) */
template <int MINB, int MODE>
int occ_mm(int block) {
  static int cached = 0;
  if (cached > 0) return cached;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused<MINB, MODE, false, 0, false>, block,
                                                    0) != cudaSuccess || nb <= 0)
    return 1;
  cached = nb;
  return nb;
}

#endif /* RAMP_FUSED_KERNEL_CUH */
