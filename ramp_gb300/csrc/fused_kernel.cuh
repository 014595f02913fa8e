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
 * Survivors of the first components can be compacted into full warps for
 * the rest of the chain (FusedArgs.split, below).
 */
#ifndef RAMP_FUSED_KERNEL_CUH
#define RAMP_FUSED_KERNEL_CUH
#include "device.cuh"
#include "launch.h"

#define FUSED_MAX_BLOCKS 32
#define FUSED_WARP_TASK 128   /* neutrons a warp claims at once */
#define FUSED_WARPS 8         /* 256-thread CTAs */
#define QWORDS 19             /* queued survivor: 16 record lanes, iidx, index, variant */
#define FULL_MASK 0xffffffffu

/* components [kb, ke) of the chain: linear blocks component by component,
 * a non-linear block whole (the split point never falls inside one).  The
 * loop counters stay warp-uniform, so descriptor loads do too. */
DI void run_range(const CompDev* __restrict__ comps, const RampBlock* __restrict__ blocks,
                  int n_blocks, int kb, int ke, Nt& n, uint32_t& ii, Rng& r, StatusDev* st,
                  bool zx) {
  for (int b = 0; b < n_blocks && !(n.die > 0.f); ++b) {
    const RampBlock B = blocks[b];
    if (B.linear) {
      for (int k = B.first; k < B.first + B.count; ++k) {
        if (k < kb || k >= ke) continue;
        if (n.die > 0.f) break;
        comp_linear(comps[k], n, ii, r, st, (NoDiff*)nullptr, zx);
      }
    } else if (B.first >= kb && B.first < ke) {
      block_nonlinear(comps, B.first, B.count, B.multi, n, ii, r, st);
    }
  }
}

/* a warp's survivor queue: QWORDS rows of 32 slots */
DI void q_put(uint32_t* q, int slot, const Nt& n, uint32_t ii, uint32_t idx, uint32_t var) {
  q[0 * 32 + slot] = __float_as_uint(n.x);   q[1 * 32 + slot] = __float_as_uint(n.y);
  q[2 * 32 + slot] = __float_as_uint(n.z);   q[3 * 32 + slot] = __float_as_uint(n.vx);
  q[4 * 32 + slot] = __float_as_uint(n.vy);  q[5 * 32 + slot] = __float_as_uint(n.vz);
  q[6 * 32 + slot] = __float_as_uint(n.px);  q[7 * 32 + slot] = __float_as_uint(n.py);
  q[8 * 32 + slot] = __float_as_uint(n.pz);  q[9 * 32 + slot] = __float_as_uint(n.p);
  q[10 * 32 + slot] = __float_as_uint(n.t);  q[11 * 32 + slot] = __float_as_uint(n.sb);
  q[12 * 32 + slot] = __float_as_uint(n.sc); q[13 * 32 + slot] = __float_as_uint(n.sd);
  q[14 * 32 + slot] = __float_as_uint(n.se); q[15 * 32 + slot] = __float_as_uint(n.die);
  q[16 * 32 + slot] = ii; q[17 * 32 + slot] = idx; q[18 * 32 + slot] = var;
}
DI void q_get(const uint32_t* q, int slot, Nt& n, uint32_t& ii, uint32_t& idx, uint32_t& var) {
  n.x = __uint_as_float(q[0 * 32 + slot]);   n.y = __uint_as_float(q[1 * 32 + slot]);
  n.z = __uint_as_float(q[2 * 32 + slot]);   n.vx = __uint_as_float(q[3 * 32 + slot]);
  n.vy = __uint_as_float(q[4 * 32 + slot]);  n.vz = __uint_as_float(q[5 * 32 + slot]);
  n.px = __uint_as_float(q[6 * 32 + slot]);  n.py = __uint_as_float(q[7 * 32 + slot]);
  n.pz = __uint_as_float(q[8 * 32 + slot]);  n.p = __uint_as_float(q[9 * 32 + slot]);
  n.t = __uint_as_float(q[10 * 32 + slot]);  n.sb = __uint_as_float(q[11 * 32 + slot]);
  n.sc = __uint_as_float(q[12 * 32 + slot]); n.sd = __uint_as_float(q[13 * 32 + slot]);
  n.se = __uint_as_float(q[14 * 32 + slot]); n.die = __uint_as_float(q[15 * 32 + slot]);
  ii = q[16 * 32 + slot]; idx = q[17 * 32 + slot]; var = q[18 * 32 + slot];
  n.wr = 0u;
}

/* the next work item of this warp: lane 0 takes it from the device counter
 * and broadcasts it.  Returns false when the work has run out. */
template <bool BATCHED>
DI bool claim(const FusedArgs& a, int lane, int& var, int64_t& start, int64_t& count) {
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(&a.st->workq, 1ull);
    t = __shfl_sync(FULL_MASK, t, 0);
    if (BATCHED) {
      const int64_t spt = (a.task_size + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK;
      const int64_t jt = (int64_t)(t / (unsigned long long)spt);
      if (jt >= a.n_tasks) return false;
      const int64_t k = (int64_t)(t % (unsigned long long)spt);
      const TaskDev T = a.tasks[jt];
      var = T.variant;
      start = T.start + k * FUSED_WARP_TASK;
      count = (int64_t)T.count - k * FUSED_WARP_TASK;
      if (count <= 0) continue;
      if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
      return true;
    } else {
      var = 0;
      start = (int64_t)t * FUSED_WARP_TASK;
      if (start >= a.single.n) return false;
      count = a.single.n - start;
      if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
      return true;
    }
  }
}

/* start neutron idx of a variant: key, carry-in, moderator */
template <int MODE>
DI void start_neutron(const FusedArgs& a, const VariantDev* V, uint32_t var, uint32_t idx,
                      bool carry, bool zx, Nt& n, Rng& r, uint32_t& ii) {
  rng_init(r, MODE, a.rng.tid_base + idx, var, a.rng.run_seed);
  const float old_sb = carry ? a.carry_sb[idx] : 0.0f;
  ii = carry ? a.carry_iidx[idx] : 0u;
  const int32_t seed = (a.rng.seed_dev && !a.tasks) ? *a.rng.seed_dev : V->seed;
  generate(V->src, n, old_sb, V->num_sim, seed, r);
  if (zx && n.p == 0.0f) n.die = 1.0f;
}

/* Without a carry buffer nothing but the tallies is observable, and every
 * later weight factor multiplies p while every tally adds p or p^2: a
 * neutron whose weight is exactly zero can only add zeros, so it is
 * retired at once (zx; the plain path, whose records are output, keeps
 * tracing it as the reference does). */

/* every neutron runs the whole chain on its lane */
template <int MODE, bool BATCHED>
DI void fused_direct(const FusedArgs& a) {
  const int lane = threadIdx.x & 31;
  const bool carry = (a.carry_sb != nullptr);
  const bool zx = !carry;
  int var;
  int64_t start, count;
  while (claim<BATCHED>(a, lane, var, start, count)) {
    const VariantDev* V = BATCHED ? a.variants + var : &a.single;
    const CompDev* comps = BATCHED ? V->comps : a.single.comps;
    for (int64_t j = lane; j < count; j += 32) {
      const uint32_t idx = (uint32_t)(start + j);
      Nt n;
      Rng r;
      uint32_t ii;
      start_neutron<MODE>(a, V, (uint32_t)var, idx, carry, zx, n, r, ii);
      run_range(comps, a.blocks, a.n_blocks, 0, a.n_comps, n, ii, r, a.st, zx);
      if (carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
    }
  }
}

/*
 * Survivor compaction (split K > 0).  Stage A (the moderator and
 * components [0, K)) runs on 32 new neutrons per pass; the components
 * after K usually see a small fraction of them (a chopper passes a few
 * per cent), which would leave most lanes of the warp idle for the rest
 * of the chain.  Survivors of stage A are therefore parked in the warp's
 * shared-memory queue until 32 are at hand, and stage B (components
 * [K, end)) runs on a full warp.  Parked survivors plus the new ones never
 * exceed 31 (a full warp is taken as soon as 32 exist), and the queue is
 * drained when the work runs out.  A neutron's record depends only on its
 * own key, so the order in which neutrons are traced changes nothing but
 * the order of tally additions.
 */
template <int MODE, bool BATCHED>
DI void fused_split(const FusedArgs& a, uint32_t* q) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int K = a.split;
  const int KEND = a.n_comps;
  const bool carry = (a.carry_sb != nullptr);
  const bool zx = !carry;
  int qn = 0;                 /* parked survivors (warp-uniform) */
  bool more = true;           /* work left to claim */
  int var = 0;
  int64_t start = 0, count = 0, j0 = 0;
  for (;;) {
    if (more && j0 >= count) {
      more = claim<BATCHED>(a, lane, var, start, count);
      j0 = 0;
    }
    if (!more && qn == 0) break;
    Nt n;
    Rng r;
    uint32_t ii = 0u, idx = 0u, var_l = 0u;
    bool live;
    int kb, ke;
    const CompDev* comps;
    if (more) {           /* stage A on (up to) 32 new neutrons */
      const VariantDev* V = BATCHED ? a.variants + var : &a.single;
      idx = (uint32_t)(start + j0 + lane);
      var_l = (uint32_t)var;
      live = j0 + lane < count;
      j0 += 32;
      if (live) start_neutron<MODE>(a, V, var_l, idx, carry, zx, n, r, ii);
      comps = BATCHED ? V->comps : a.single.comps;
      kb = 0;
      ke = K;
    } else {              /* drain: the parked survivors run stage B */
      live = lane < qn;
      if (live) {
        q_get(q, lane, n, ii, idx, var_l);
        rng_init(r, MODE, a.rng.tid_base + idx, var_l, a.rng.run_seed);
      }
      __syncwarp();
      qn = 0;
      comps = BATCHED ? a.variants[var_l].comps : a.single.comps;
      kb = K;
      ke = KEND;
    }
    for (;;) {
      if (live) run_range(comps, a.blocks, a.n_blocks, kb, ke, n, ii, r, a.st, zx);
      if (kb == K) break;             /* stage B finished */
      /* end of stage A */
      const bool alive = live && !(n.die > 0.f);
      if (live && !alive && carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
      const unsigned m = __ballot_sync(FULL_MASK, alive);
      const int S = __popc(m);
      if (qn + S < 32) {
        if (alive) q_put(q, qn + __popc(m & lt), n, ii, idx, var_l);
        __syncwarp();
        qn += S;
        live = false;
        break;
      }
      /* a full warp: the lanes without a survivor take parked ones */
      if (!alive) {
        q_get(q, qn - 1 - __popc(~m & lt), n, ii, idx, var_l);
        rng_init(r, MODE, a.rng.tid_base + idx, var_l, a.rng.run_seed);
        if (BATCHED) comps = a.variants[var_l].comps;
      }
      __syncwarp();
      qn -= 32 - S;
      live = true;
      kb = K;
      ke = KEND;
    }
    if (live && carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
  }
}

template <int MINB, int MODE, bool BATCHED, bool SPLIT>
__global__ void __launch_bounds__(256, MINB) k_fused(const FusedArgs a) {
  if constexpr (SPLIT) {
    __shared__ uint32_t qbuf[FUSED_WARPS * QWORDS * 32];
    fused_split<MODE, BATCHED>(a, qbuf + (threadIdx.x >> 5) * (QWORDS * 32));
  } else {
    fused_direct<MODE, BATCHED>(a);
  }
}

/* one register cap and keying mode: the four layouts (single/batched,
 * direct/split) */
template <int MINB, int MODE>
cudaError_t launch_mm(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  const bool b = a.variants != nullptr, sp = a.split > 0;
  if (b) {
    if (sp) k_fused<MINB, MODE, true, true><<<grid, block, 0, s>>>(a);
    else k_fused<MINB, MODE, true, false><<<grid, block, 0, s>>>(a);
  } else {
    if (sp) k_fused<MINB, MODE, false, true><<<grid, block, 0, s>>>(a);
    else k_fused<MINB, MODE, false, false><<<grid, block, 0, s>>>(a);
  }
  return cudaGetLastError();
}

template <int MINB, int MODE>
int occ_mm(int block) {
  static int cached = 0;
  if (cached > 0) return cached;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused<MINB, MODE, false, false>, block,
                                                    0) != cudaSuccess || nb <= 0)
    return 1;
  cached = nb;
  return nb;
}

#endif /* RAMP_FUSED_KERNEL_CUH */
