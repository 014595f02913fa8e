/*
 * adjoint.cu — gradients of a detector-histogram loss with respect to
 * weight parameters (ramp_adjoint).  Each thread replays one neutron from
 * its counter-based RNG key through the same device functions as the
 * forward paths, instantiated with an AdjDiff context that accumulates
 * d log p / d theta and contributes dL/dH_bin * p * d log p / d theta at the
 * loss detector.  The replay is the checkpoint: a neutron's state at every
 * component boundary is recomputed exactly, nothing per neutron is stored.
 * Only neutrons the loss detector counts carry a term, so a first pass
 * (no derivatives) lists their indices and the second replays just those
 * with the derivative context.  When the chain starts with a chopper run
 * (lookahead.h), the first pass is split in two: every neutron's first draw
 * and the speed look-ahead, keeping the indices of those that may pass (the
 * others add nothing to a tally and are never counted), then the whole
 * chain for the kept ones, 32 to a warp, each regenerated from its key (the
 * same operations, so the same neutron).
 */
#include "device.cuh"
#include "launch.h"
#include "lookahead.h"

/* one neutron through the chain with context D */
template <class D, int MODE>
DI void adj_trace(const AdjointArgs& a, uint32_t i, D& dx) {
  Nt n;
  Rng r;
  rng_init(r, MODE, a.rng.tid_base + i, 0u, a.rng.run_seed, a.rng.one);
  uint32_t ii = 0;
  generate<D>(a.src, n, 0.0f, a.num_sim, a.rng.seed_dev ? *a.rng.seed_dev : a.seed, r, &dx);
  /* a zero-weight neutron contributes dL/dH * p * dlog p = 0: retired */
  if (n.p == 0.0f) n.die = 1.0f;
  for (int b = 0; b < a.n_blocks && !(n.die > 0.f); ++b) {
    const RampBlock B = a.blocks[b];
    if (B.linear) {
      for (int k = B.first; k < B.first + B.count; ++k) {
        if (n.die > 0.f) break;
        comp_linear<D>(a.comps[k], n, ii, r, a.st, &dx, true);
      }
    } else {
      block_nonlinear<D>(a.comps, B.first, B.count, B.multi, n, ii, r, a.st, &dx);
    }
  }
}

/* pass 1: every neutron (KEPT: the neutrons of the kept list), the
 * indices the loss detector counts (with TALLY, also the forward
 * histograms) */
template <int MODE, bool TALLY, bool KEPT>
__global__ void __launch_bounds__(256) k_adjoint_record(const AdjointArgs a) {
  int64_t m = a.n;
  if (KEPT) {
    m = (int64_t)*a.keep_count;
    if (m > a.list_cap) m = a.list_cap;
  }
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = KEPT ? a.keep[j] : (uint32_t)j;
    RecorderT<TALLY> dx;
    dx.idx = i;
    dx.done = false;
    dx.list = a.list;
    dx.count = a.list_count;
    dx.cap = a.list_cap;
    adj_trace<RecorderT<TALLY>, MODE>(a, i, dx);
  }
}

/* the speed table of the keep pass (lookahead.h) lives after the three
 * counters of the index lists */
DI uint32_t* adjoint_speed_tab(const AdjointArgs& a) {
  return reinterpret_cast<uint32_t*>(a.list_count + 3);
}

/* pass 1, before the keep pass, for a flat or MCont source: the speed
 * table, SPEED_CELLS / 256 CTAs */
__global__ void __launch_bounds__(256) k_adjoint_table(const AdjointArgs a) {
  __shared__ SpeedTab T;
  __shared__ int blocked[SPEED_RUN_MAX];
  speed_tab_build(adjoint_speed_tab(a), &T, blocked, a.comps, a.cull, a.src.p,
                  (int)blockIdx.x);
}

/* pass 1, first half: for every neutron its first draw (the energy, hence
 * the speed) and the speed look-ahead (speed_tab_blocks with the table of
 * k_adjoint_table; with a source other than flat or MCont the moderator
 * and the full look-ahead); the indices of those it keeps are appended to
 * a.keep (warp_list_add) */
template <int MODE>
__global__ void __launch_bounds__(256) k_adjoint_keep(const AdjointArgs a) {
  const bool speed = a.src.kind == RAMP_SRC_FLAT || a.src.kind == RAMP_SRC_CONT;
  __shared__ SpeedTab tab;
  if (speed) speed_tab_load(&tab, adjoint_speed_tab(a));
  const int lane = threadIdx.x & 31;
  __shared__ uint32_t stage[256 / 32][64];
  int held = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  for (int64_t base = i0; base < a.n; base += stride) {   /* warp-uniform */
    const int64_t i = base + lane;
    bool kept = false;
    if (i < a.n) {
      Nt n;
      Rng r;
      rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, 0u, a.rng.run_seed, a.rng.one);
      const int32_t seed = a.rng.seed_dev ? *a.rng.seed_dev : a.seed;
      if (speed) {
        n.sb = (float)seed + 0.0f;      /* generate's first draw */
        kept = !speed_tab_blocks(tab, draw_word(n, r));
      } else {
        generate<TallyOnly, true, false>(a.src, n, 0.0f, a.num_sim, seed, r);
        kept = !chopper_run_blocks(a.comps, 0, a.cull, n.x, n.y, n.z, n.vx, n.vy, n.vz, n.t);
      }
    }
    warp_list_add(kept, (uint32_t)i, stage[threadIdx.x >> 5], held, a.keep_count, a.keep,
                  a.list_cap);
  }
  warp_list_flush(stage[threadIdx.x >> 5], held, a.keep_count, a.keep, a.list_cap);
}

/* pass 2: the recorded neutrons, replayed with d log p / d theta */
template <int MODE>
__global__ void __launch_bounds__(256) k_adjoint(const AdjointArgs a) {
  int64_t m = (int64_t)*a.list_count;
  if (m > a.list_cap) m = a.list_cap;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    AdjDiff dx;
    dx.reset(a.nslot, a.grad, a.lr);
    adj_trace<AdjDiff, MODE>(a, a.list[j], dx);
  }
}

/* passes: bit 1 record (bit 4: with tallies), bit 2 replay */
cudaError_t launch_adjoint(const AdjointArgs& a, int grid, int passes, cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.n <= 0) return cudaSuccess;
  if (passes & 1) {
    cudaError_t e = cudaMemsetAsync(a.list_count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const bool t = (passes & 4) != 0;
    if (a.cull > 0) {          /* keep, then trace the kept neutrons */
      e = cudaMemsetAsync(a.keep_count, 0, sizeof(unsigned long long), s);
      if (e != cudaSuccess) return e;
      if (a.src.kind == RAMP_SRC_FLAT || a.src.kind == RAMP_SRC_CONT)
        k_adjoint_table<<<SPEED_CELLS / 256, 256, 0, s>>>(a);
      if (a.rng.mode == 0) {
        k_adjoint_keep<0><<<grid, 256, 0, s>>>(a);
        if (t) k_adjoint_record<0, true, true><<<grid, 256, 0, s>>>(a);
        else k_adjoint_record<0, false, true><<<grid, 256, 0, s>>>(a);
      } else {
        k_adjoint_keep<1><<<grid, 256, 0, s>>>(a);
        if (t) k_adjoint_record<1, true, true><<<grid, 256, 0, s>>>(a);
        else k_adjoint_record<1, false, true><<<grid, 256, 0, s>>>(a);
      }
    } else if (a.rng.mode == 0) {
      if (t) k_adjoint_record<0, true, false><<<grid, 256, 0, s>>>(a);
      else k_adjoint_record<0, false, false><<<grid, 256, 0, s>>>(a);
    } else {
      if (t) k_adjoint_record<1, true, false><<<grid, 256, 0, s>>>(a);
      else k_adjoint_record<1, false, false><<<grid, 256, 0, s>>>(a);
    }
  }
  if (passes & 2) {
    if (a.rng.mode == 0) k_adjoint<0><<<grid, 256, 0, s>>>(a);
    else k_adjoint<1><<<grid, 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}
