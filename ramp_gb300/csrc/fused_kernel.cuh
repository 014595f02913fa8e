/*
 * fused_kernel.cuh — the fused path: one persistent kernel runs the whole chain
 * (moderator, every block and component) with each neutron in registers;
 * nothing but the tallies touches HBM.  Work is claimed per warp: lane 0
 * takes the next item (128 neutrons of one variant) from a device counter
 * and broadcasts it, so warps never wait on each other (no CTA barrier).
 * Many instrument variants with uneven neutron counts share one launch
 * (BATCHED): grid row y traces variant y from its own work counter, so the
 * variant index is blockIdx.y — uniform by construction, which keeps the
 * descriptor addresses in uniform registers as in a one-instrument launch
 * (an index read per warp from a task list made the kernel 5-8x slower).
 * Component descriptors are read through the read-only cache (every lane
 * of a warp reads the same address).  The kernel is instantiated per RNG keying mode
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
#include "lookahead.h"

#define FUSED_MAX_BLOCKS 32
/* the mesh walk (PHASE 4) holds only the ray and the walk state: it is
 * compiled for more resident CTAs per SM than the other phases (40
 * registers at 6 CTAs of 256 threads, against 64 at 4), and its
 * single-instrument grid fills that occupancy */
#ifndef WALK_MINB
#define WALK_MINB 6
#endif
/* the walk hands waiting rays to idle lanes once this many of a warp's 32
 * lanes are idle (or when none is left walking) */
#ifndef WALK_REFILL
#define WALK_REFILL 8
#endif
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
 * buffer (no atomics) and finish in PHASE 2.  PHASE 3: stage A of a launch
 * split before component 0 (the moderator and the chopper look-ahead),
 * compiled without the component code.  The bounds of both loops are kernel parameters, so the loop
 * counters and descriptor addresses stay warp-uniform.
 */
template <int MINB, int MODE, bool BATCHED, int PHASE, int KS>
__global__ void __launch_bounds__(256, PHASE == 4 ? WALK_MINB : MINB)
k_fused(const FusedArgs a);

/* PHASE 2: the survivors of stage A through components [split, end).
 * Stage A leaves the survivors of work item t at slots [128 t, 128 t +
 * cnt[t]) (batched: item item_off + t of its variant's row); a warp claims
 * up to SURV_GROUP items at a time (fewer when there are too few items to
 * give every warp of the grid two claims) and deals their survivors out 32
 * to a pass.
 * A survivor is keyed by its own index and variant, so it continues
 * exactly where stage A left it. */
#define SURV_GROUP 32   /* one work item per lane */

template <int MODE, int KS>
DI void walk_end(const FusedArgs& a, const CompDev* __restrict__ comps, int K, int64_t slot,
                 const MeshRec& w, int k, bool zx, bool carry);

/* the result of a finished mesh walk (k = 0: the walk ended, -1: the stack
 * overflowed, -2: the ray missed the mesh box), kept beside the survivor's
 * record for PHASE 5 */
DI void walk_store(const FusedArgs& a, int64_t slot, const MeshRec& r, int k) {
  uint32_t* wp = a.surv + slot;
  const int64_t cap = a.surv_cap;
  const unsigned long long cb = (unsigned long long)__double_as_longlong(r.chord);
  wp[18 * cap] = __float_as_uint(r.o3);
  wp[19 * cap] = __float_as_uint(r.o7);
  wp[20 * cap] = (uint32_t)cb;
  wp[21 * cap] = (uint32_t)(cb >> 32);
  wp[22 * cap] = r.num_intersections;
  wp[23 * cap] = (uint32_t)k;
}

/* the item of the current group that holds survivor q: the last item whose
 * first survivor (excl, one item per lane, non-decreasing over the lanes)
 * is at or before q, by binary search over the lanes; *base is that first
 * survivor.  Every lane of the warp takes part. */
DI int surv_item(int excl, int q, int* base) {
  int lo = 0;
  for (int step = 16; step >= 1; step >>= 1) {
    const int e = __shfl_sync(FULL_MASK, excl, lo + step);
    if (e <= q) lo += step;
  }
  *base = __shfl_sync(FULL_MASK, excl, lo);
  return lo;
}
template <int MODE, bool BATCHED, int KS, bool FINISH = false>
DI void fused_tail(const FusedArgs& a) {
  constexpr bool EXT = KS == 1, MESH = KS != 0;
  const int lane = threadIdx.x & 31;
  const bool carry = (a.carry_sb != nullptr);
  const bool zx = !carry;
  const int K = a.split;
  const int64_t cap = a.surv_cap;
  /* this launch's (batched: this row's variant's) work items */
  const int var = BATCHED ? (int)blockIdx.y : a.var_key;
  const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
  const int64_t item0 = BATCHED ? V->item_off : 0;
  int64_t n_items = BATCHED ? (V->n + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK : a.surv_items;
  if (BATCHED && item0 + n_items > a.surv_items) {   /* host sized the buffer for every row */
    if (lane == 0) raise_flag(a.st, RAMP_F_WORKQ);
    return;
  }
  /* after the lean stage A only the items of the listed histories hold
     survivors (their number in workq_c, written by k_speed_keep) */
  if (!FINISH && KS == 0 && K == 0 && a.cull > 0) {
    const int64_t used = ((int64_t)a.workq_c[BATCHED ? var : 0] + FUSED_WARP_TASK - 1) /
                         FUSED_WARP_TASK;
    if (used < n_items) n_items = used;
  }
  /* items per grab: about two grabs per warp of the grid, or (after the
     lean stage A of one instrument, whose survivors are counted) enough
     items for about 32 survivors when that is more; at most one item per
     lane */
  int64_t per = n_items / (2 * (int64_t)gridDim.x * (blockDim.x >> 5));
  if (!FINISH && !BATCHED && KS == 0 && K == 0 && a.cull > 0) {
    const int64_t tot = (int64_t)a.st->surv;
    const int64_t fill = tot > 0 ? (32 * n_items + tot - 1) / tot : SURV_GROUP;
    if (fill > per) per = fill;
  }
  const int G = per < 1 ? 1 : (per > SURV_GROUP ? SURV_GROUP : (int)per);
  const CompDev* __restrict__ comps = V->comps;
  unsigned long long* const q_b = (FINISH ? a.workq_c : a.workq_b) + (BATCHED ? var : 0);
  for (;;) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(q_b, 1ull);
    g = __shfl_sync(FULL_MASK, g, 0);
    const int64_t t0 = (int64_t)g * G;
    if (t0 >= n_items) break;
    const int c = (lane < G && t0 + lane < n_items) ? (int)a.surv_cnt[item0 + t0 + lane] : 0;
    int incl = c;
    for (int d = 1; d < SURV_GROUP; d <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, incl, d);
      if (lane >= d) incl += y;
    }
    const int excl = incl - c;
    const int total = __shfl_sync(FULL_MASK, incl, SURV_GROUP - 1);
    for (int q0 = 0; q0 < total; q0 += 32) {
      const int q = q0 + lane;
      int base = 0;
      const int item = surv_item(excl, q, &base);
      if (q >= total) continue;
      const int64_t s = (item0 + t0 + item) * FUSED_WARP_TASK + (q - base);
      const uint32_t* w = a.surv + s;
      if constexpr (FINISH) {   /* PHASE 5: the rest of the chain after a mesh walk */
        MeshRec rec;
        rec.o3 = __uint_as_float(w[18 * cap]);
        rec.o7 = __uint_as_float(w[19 * cap]);
        rec.chord = __longlong_as_double(
            (long long)(((unsigned long long)w[21 * cap] << 32) | (unsigned long long)w[20 * cap]));
        rec.num_intersections = w[22 * cap];
        walk_end<MODE, KS>(a, comps, K, s, rec, (int)w[23 * cap], zx, carry);
        continue;
      }
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
      const uint32_t idx = w[16 * cap];
      Rng r;
      rng_init(r, MODE, a.rng.tid_base + idx, w[17 * cap], a.rng.run_seed, a.rng.one);
      for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
        const RampBlock B = a.blocks[b];
        const int e = B.first + B.count;
        if (e <= K) continue;
        if (B.linear) {
          for (int k = B.first > K ? B.first : K; k < e; ++k) {
            if (n.die > 0.f) break;
            comp_linear<TallyOnly, EXT, MESH>(comps[k], n, ii, r, a.st, (TallyOnly*)nullptr, zx);
          }
        } else {
          block_nonlinear<TallyOnly, EXT, MESH>(comps, B.first, B.count, B.multi, n, ii, r, a.st);
        }
      }
      if (carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
    }
  }
}

/* a neutron whose walk through the GMesh component K is over (k = 0: the
 * walk ended, -1: the stack overflowed, -2: the ray missed the mesh box):
 * read it back from its survivor record, bring it into K's frame again
 * (the same operations give the same values), take the walk's records, then
 * the rest of comp_linear of K and the components after it */
template <int MODE, int KS>
DI void walk_end(const FusedArgs& a, const CompDev* __restrict__ comps, int K, int64_t slot,
                 const MeshRec& w, int k, bool zx, bool carry) {
  constexpr bool EXT = KS == 1, MESH = KS != 0;
  const int64_t cap = a.surv_cap;
  const uint32_t* wp = a.surv + slot;
  Nt n;
  n.x = __uint_as_float(wp[0 * cap]);   n.y = __uint_as_float(wp[1 * cap]);
  n.z = __uint_as_float(wp[2 * cap]);   n.vx = __uint_as_float(wp[3 * cap]);
  n.vy = __uint_as_float(wp[4 * cap]);  n.vz = __uint_as_float(wp[5 * cap]);
  n.px = __uint_as_float(wp[6 * cap]);  n.py = __uint_as_float(wp[7 * cap]);
  n.pz = __uint_as_float(wp[8 * cap]);  n.p = __uint_as_float(wp[9 * cap]);
  n.t = __uint_as_float(wp[10 * cap]);  n.sb = __uint_as_float(wp[11 * cap]);
  n.sc = __uint_as_float(wp[12 * cap]); n.sd = __uint_as_float(wp[13 * cap]);
  n.se = __uint_as_float(wp[14 * cap]);
  n.die = 0.0f;
  n.wr = 0u;
  uint32_t ii = wp[15 * cap];
  const uint32_t idx = wp[16 * cap];
  Rng r;
  rng_init(r, MODE, a.rng.tid_base + idx, wp[17 * cap], a.rng.run_seed, a.rng.one);
  const CompDev& cK = comps[K];
  transform<false>(cK, n);
  Is s;
  is_reset(s);
  if (k == 0 && mesh_end(cK, n, s, w)) ii = cK.idx;
  if (len3(ip2(s)) == 0.0f && cK.restore == 0) set_die(n, 1.f);
  if (ii == cK.idx && !(n.die > 0.f))
    scatter<TallyOnly, EXT, MESH>(cK, n, s, ii, r, a.st, (TallyOnly*)nullptr, zx);
  if (zx && n.p == 0.0f) set_die(n, 1.0f);
  else if (!(n.die > 0.f)) untransform<false>(cK, n);
  for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
    const RampBlock B = a.blocks[b];
    const int e = B.first + B.count;
    if (e <= K + 1) continue;
    if (B.linear) {
      for (int j = B.first > K + 1 ? B.first : K + 1; j < e; ++j) {
        if (n.die > 0.f) break;
        comp_linear<TallyOnly, EXT, MESH>(comps[j], n, ii, r, a.st, (TallyOnly*)nullptr, zx);
      }
    } else {
      block_nonlinear<TallyOnly, EXT, MESH>(comps, B.first, B.count, B.multi, n, ii, r, a.st);
    }
  }
  if (carry) { a.carry_sb[idx] = n.sb; a.carry_iidx[idx] = ii; }
}

/* PHASE 4: stage B of a launch split before a GMesh component K (a linear
 * block's), for chains where the walk through the mesh hierarchy is most of
 * the work.  Walk lengths differ a lot between rays (a ray outside the mesh
 * box has none), so with one ray per lane a warp runs at a few lanes.  Here
 * each lane walks its ray one node visit or one triangle per pass (the warp
 * runs the kind more of its lanes wait for), and a lane whose walk is over
 * stores its result beside the survivor's record and takes the next waiting
 * survivor; the warp claims the next group of work items as soon as every
 * survivor of the current one is taken.  PHASE 5 then finishes every
 * survivor 32 to a warp (the rest of component K and the components after
 * it): kept out of the walk's loop, that code would otherwise make the loop
 * spill (1.5 KB of spill stores per thread at 64 registers; none without
 * it).  Every neutron goes through the same operations as in PHASE 2 (the
 * records and the chord do not depend on the order in which triangles are
 * visited). */
template <int MODE, bool BATCHED, int KS>
DI void fused_tail_walk(const FusedArgs& a) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int K = a.split;
  const int64_t cap = a.surv_cap;
  const int var = BATCHED ? (int)blockIdx.y : a.var_key;
  const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
  const int64_t item0 = BATCHED ? V->item_off : 0;
  const int64_t n_items = BATCHED ? (V->n + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK : a.surv_items;
  if (BATCHED && item0 + n_items > a.surv_items) {
    if (lane == 0) raise_flag(a.st, RAMP_F_WORKQ);
    return;
  }
  const CompDev* __restrict__ comps = V->comps;
  const CompDev& cK = comps[K];
  unsigned long long* const q_b = a.workq_b + (BATCHED ? var : 0);
  /* the current group of work items (warp-uniform) */
  int64_t t0 = 0;
  int c = 0, excl = 0, total = 0, handed = 0;
  bool groups_left = true;
  /* this lane's walk: only the ray and the walk state stay live while it
     runs; the neutron is read back from its survivor record when it ends */
  bool walking = false;
  int64_t slot = 0;
  MeshWalk w;
  /* this thread's column of the shared-memory part of the walk stack */
  int* const sstack = reinterpret_cast<int*>(ramp_dyn_smem) + threadIdx.x;
  for (;;) {
    /* hand the waiting survivors to the idle lanes (a lane whose ray misses
       the mesh box finishes it at once and is idle again) */
    for (;;) {
      const unsigned m = __ballot_sync(FULL_MASK, !walking);
      if (m == 0u) break;
      if (handed >= total) {
        if (!groups_left) break;
        unsigned long long g = 0;
        if (lane == 0) g = atomicAdd(q_b, 1ull);
        g = __shfl_sync(FULL_MASK, g, 0);
        t0 = (int64_t)g * SURV_GROUP;
        handed = 0;
        if (t0 >= n_items) {
          groups_left = false;
          c = 0; excl = 0; total = 0;
          break;
        }
        c = (lane < SURV_GROUP && t0 + lane < n_items) ? (int)a.surv_cnt[item0 + t0 + lane] : 0;
        int incl = c;
        for (int d = 1; d < SURV_GROUP; d <<= 1) {
          const int y = __shfl_up_sync(FULL_MASK, incl, d);
          if (lane >= d) incl += y;
        }
        excl = incl - c;
        total = __shfl_sync(FULL_MASK, incl, SURV_GROUP - 1);
        continue;
      }
      const int qk = handed + __popc(m & lt);
      int base = 0;
      const int item = surv_item(excl, qk, &base);
      handed = (handed + __popc(m) < total) ? handed + __popc(m) : total;
      if (!walking && qk < total) {
        slot = (item0 + t0 + item) * FUSED_WARP_TASK + (qk - base);
        const uint32_t* wp = a.surv + slot;
        Nt ray;                           /* position and velocity suffice for the walk */
        ray.x = __uint_as_float(wp[0 * cap]);  ray.y = __uint_as_float(wp[1 * cap]);
        ray.z = __uint_as_float(wp[2 * cap]);  ray.vx = __uint_as_float(wp[3 * cap]);
        ray.vy = __uint_as_float(wp[4 * cap]); ray.vz = __uint_as_float(wp[5 * cap]);
        transform<false>(cK, ray);        /* comp_linear of component K */
        if (mesh_begin(cK, ray, w)) walking = true;
        else walk_store(a, slot, mesh_rec(w), -2);
      }
    }
    const bool more = groups_left || handed < total;   /* survivors still waiting */
    if (!more && !__any_sync(FULL_MASK, walking)) break;
    /* walk until WALK_REFILL lanes are idle (or, with nothing left
       to hand out, until every walk is over).  Each pass runs one kind of
       work, the kind more lanes wait for: a triangle of each lane's pending
       leaf range, or an inner node of each lane without one */
    for (;;) {
      const bool wt = walking && w.tb < w.te;
      const unsigned bt = __ballot_sync(FULL_MASK, wt);
      const unsigned bn = __ballot_sync(FULL_MASK, walking && !wt);
      bool ok = true;
      if (__popc(bt) >= __popc(bn)) {
        if (wt) mesh_tri(cK, w, w.tb++);
      } else if (walking && !wt) {
        ok = mesh_visit(cK, w, a.st, sstack, (int)blockDim.x);
      }
      if (walking && (!ok || mesh_walk_over(w))) {
        walking = false;
        walk_store(a, slot, mesh_rec(w), ok ? 0 : -1);
      }
      const int idle = __popc(__ballot_sync(FULL_MASK, !walking));
      if (idle == 32 || (more && idle >= WALK_REFILL)) break;
    }
  }
}

template <int MINB, int MODE, bool BATCHED, int PHASE, int KS>
__global__ void __launch_bounds__(256, PHASE == 4 ? WALK_MINB : MINB)
k_fused(const FusedArgs a) {
  constexpr bool EXT = KS == 1, MESH = KS != 0;
  if constexpr (PHASE == 2 || PHASE == 5) {
    fused_tail<MODE, BATCHED, KS, PHASE == 5>(a);
    return;
  } else if constexpr (PHASE == 4) {
    fused_tail_walk<MODE, BATCHED, KS>(a);
    return;
  } else {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    constexpr bool STAGE_A = PHASE == 1 || PHASE == 3;
    const int KE = PHASE == 3 ? 0 : (PHASE == 1 ? a.split : a.n_comps);
    const int var = BATCHED ? (int)blockIdx.y : a.var_key;
    const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
    const int64_t item0 = BATCHED ? V->item_off : 0;
    /* the lean stage A traces the histories the speed look-ahead listed
       (k_speed_keep in fused.cu: their indices in word 18 of the survivor
       slots, their number in workq_c); the other phases every history */
    const uint32_t* __restrict__ listed = a.surv + (size_t)18 * a.surv_cap + item0 * FUSED_WARP_TASK;
    int64_t n_work = V->n;
    if (PHASE == 3) {
      const int64_t m = (int64_t)a.workq_c[BATCHED ? var : 0];
      if (m < n_work) n_work = m;
    }
    /* batched: CTAs past what this row's variant can use leave at once */
    if (BATCHED && (int64_t)blockIdx.x * (blockDim.x / 32) * FUSED_WARP_TASK >= n_work) return;
    unsigned long long* const q_a = a.workq + (BATCHED ? var : 0);
    const bool priv = PHASE == 0 && !BATCHED && a.priv_floats > 0;
    if (priv) {                   /* the CTA's private tallies start at zero */
      for (int k = threadIdx.x; k < a.priv_floats; k += blockDim.x) ramp_dyn_smem[k] = 0.0f;
      __syncthreads();
    }
    for (;;) {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(q_a, 1ull);
      t = __shfl_sync(FULL_MASK, t, 0);
      const int64_t start = (int64_t)t * FUSED_WARP_TASK;
      if (start >= n_work) break;
      int64_t count = n_work - start;
      if (count > FUSED_WARP_TASK) count = FUSED_WARP_TASK;
      const CompDev* __restrict__ comps = V->comps;
      const int32_t num_sim = V->num_sim;
      const int32_t seed = (a.rng.seed_dev && !BATCHED) ? *a.rng.seed_dev : V->seed;
      const bool carry = (a.carry_sb != nullptr);
      const bool zx = !carry;
      int kept = 0;      /* PHASE 1: survivors of this item so far (warp-uniform) */
      /* PHASE 1 keeps the whole warp in the loop for the ballot */
      const int jend = STAGE_A ? (int)((count + 31) & ~31ll) : (int)count;
      for (int j = lane; j < jend; j += 32) {
        const bool live = j < count;
        const int64_t i = (PHASE == 3 && live) ? (int64_t)listed[start + j] : start + j;
        Nt n;
        Rng r;
        uint32_t ii = 0u;
        if (live) {
          rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed,
                   a.rng.one);
          const float old_sb = carry ? a.carry_sb[i] : 0.0f;
          ii = carry ? a.carry_iidx[i] : 0u;
          /* the lean stage A (core kinds: flat or MCont source) weighs a
             history only once the look-ahead has kept it */
          generate<TallyOnly, EXT, PHASE != 3>(V->src, n, old_sb, num_sim, seed, r);
          if (PHASE != 3 && zx && n.p == 0.0f) n.die = 1.0f;
          if constexpr (PHASE != 3) {
            for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
              const RampBlock B = a.blocks[b];
              if (PHASE == 1 && B.first >= KE) break;
              if (B.linear) {
                const int e = (PHASE == 1 && B.first + B.count > KE) ? KE : B.first + B.count;
                for (int k = B.first; k < e; ++k) {
                  if (n.die > 0.f) break;
                  comp_linear<TallyOnly, EXT, MESH>(comps[k], n, ii, r, a.st, (TallyOnly*)nullptr,
                                                    zx);
                }
              } else {
                block_nonlinear<TallyOnly, EXT, MESH>(comps, B.first, B.count, B.multi, n, ii, r,
                                                      a.st);
              }
            }
          }
          /* the chopper look-ahead: a neutron that certainly cannot pass
             the choppers after the split adds nothing to any tally */
          if (STAGE_A && zx && a.cull > 0 && !(n.die > 0.f) &&
              chopper_run_blocks(comps, KE, a.cull, n.x, n.y, n.z, n.vx, n.vy, n.vz, n.t))
            n.die = 1.0f;
          if (PHASE == 3 && !(n.die > 0.f)) {
            n.p = source_weight<TallyOnly>(V->src, n.p, num_sim);
            if (zx && n.p == 0.0f) n.die = 1.0f;
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
        const int64_t s = (item0 + (int64_t)t) * FUSED_WARP_TASK + rank;   /* rank < 128 */
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
      if (STAGE_A && lane == 0 && item0 + (int64_t)t < a.surv_items)
        a.surv_cnt[item0 + t] = (uint32_t)kept;
      /* the lean stage A's survivors in all (stage B sizes its claims by it) */
      if (PHASE == 3 && !BATCHED && lane == 0 && kept > 0)
        atomicAdd(&a.st->surv, (unsigned long long)kept);
    }
    if (priv) {                   /* merge the private tallies, nonzero bins only */
      __syncthreads();
      const CompDev* __restrict__ comps = V->comps;
      for (int j = 0; j < a.n_comps; ++j) {
        const int off = comps[j].priv_off;
        if (off < 0) continue;
        const int64_t len = comps[j].tally_len;
        float* const h = comps[j].tally;
        float* const he = comps[j].tally_err;
        for (int64_t k = threadIdx.x; k < len; k += blockDim.x) {
          const float v = ramp_dyn_smem[off + k];
          if (v != 0.0f) atomicAdd(h + k, v);
          if (he) {
            const float w = ramp_dyn_smem[off + len + k];
            if (w != 0.0f) atomicAdd(he + k, w);
          }
        }
      }
    }
  }
}

/* one launch of one instantiation; each is compiled in a translation unit
 * of its own (fused_inst.cu, built once per template argument set) and the
 * sequencing of phases lives in fused.cu */
template <int MINB, int MODE, bool BATCHED, int PHASE, int KS>
cudaError_t launch_phase(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if constexpr (PHASE == 4 && !BATCHED) {   /* the walk's own occupancy: CTAs x SMs */
    static int cached[2] = {0, 0};         /* 256- and 128-thread CTAs */
    int& nb = cached[block == 128 ? 1 : 0];
    if (nb == 0) {
      int dev = 0, sms = 0, per_sm = 0;
      if (cudaGetDevice(&dev) == cudaSuccess &&
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &per_sm, k_fused<MINB, MODE, false, 4, KS>, block,
              (size_t)RAMP_BVH_SSTACK * block * sizeof(int)) == cudaSuccess &&
          per_sm > 0)
        nb = sms * per_sm;
      else
        nb = -1;
    }
    if (nb > grid) grid = nb;
  }
  const dim3 g((unsigned)grid, BATCHED ? (unsigned)a.n_variants : 1u);
  size_t smem = 0;
  if (PHASE == 0 && !BATCHED && a.priv_floats > 0)
    smem = (size_t)a.priv_floats * sizeof(float);    /* at most 48 KB: no attribute */
  if (PHASE == 4) smem = (size_t)RAMP_BVH_SSTACK * block * sizeof(int);   /* 16 KB */
  k_fused<MINB, MODE, BATCHED, PHASE, KS><<<g, block, smem, s>>>(a);
  return cudaGetLastError();
}

/* occupancy of the whole-chain kernel at this register cap (CTAs per SM) */
template <int MINB, int MODE>
int occ_mm(int block) {
  static int cached[2] = {0, 0};     /* 256- and 128-thread CTAs */
  const int slot = block == 128 ? 1 : 0;
  if (cached[slot] > 0) return cached[slot];
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused<MINB, MODE, false, 0, 0>, block,
                                                    0) != cudaSuccess || nb <= 0)
    return 1;
  cached[slot] = nb;
  return nb;
}

#endif /* RAMP_FUSED_KERNEL_CUH */
