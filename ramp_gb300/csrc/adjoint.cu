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
 * with the derivative context.  The first pass retires after the moderator
 * the neutrons that certainly cannot pass the chopper run the chain starts
 * with (lookahead.h): they add nothing to a tally and are never counted.
 */
#include "device.cuh"
#include "launch.h"
#include "lookahead.h"

/* one neutron through the chain with context D (CULL: with the chopper
 * look-ahead after the moderator) */
template <class D, int MODE, bool CULL = false>
DI void adj_trace(const AdjointArgs& a, uint32_t i, D& dx) {
  Nt n;
  Rng r;
  rng_init(r, MODE, a.rng.tid_base + i, 0u, a.rng.run_seed);
  uint32_t ii = 0;
  generate<D>(a.src, n, 0.0f, a.num_sim, a.rng.seed_dev ? *a.rng.seed_dev : a.seed, r, &dx);
  /* a zero-weight neutron contributes dL/dH * p * dlog p = 0: retired */
  if (n.p == 0.0f) n.die = 1.0f;
  if (CULL && a.cull > 0 && !(n.die > 0.f) &&
      chopper_run_blocks(a.comps, 0, a.cull, n.x, n.y, n.z, n.vx, n.vy, n.vz, n.t))
    n.die = 1.0f;
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

/* pass 1: every neutron, the indices the loss detector counts (with TALLY,
 * also the forward histograms) */
template <int MODE, bool TALLY>
__global__ void __launch_bounds__(256) k_adjoint_record(const AdjointArgs a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    RecorderT<TALLY> dx;
    dx.idx = (uint32_t)i;
    dx.done = false;
    dx.list = a.list;
    dx.count = a.list_count;
    dx.cap = a.list_cap;
    adj_trace<RecorderT<TALLY>, MODE, true>(a, (uint32_t)i, dx);
  }
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
  if (a.n <= 0) return cudaSuccess;
  if (passes & 1) {
    cudaError_t e = cudaMemsetAsync(a.list_count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const bool t = (passes & 4) != 0;
    if (a.rng.mode == 0) {
      if (t) k_adjoint_record<0, true><<<grid, 256, 0, s>>>(a);
      else k_adjoint_record<0, false><<<grid, 256, 0, s>>>(a);
    } else {
      if (t) k_adjoint_record<1, true><<<grid, 256, 0, s>>>(a);
      else k_adjoint_record<1, false><<<grid, 256, 0, s>>>(a);
    }
  }
  if (passes & 2) {
    if (a.rng.mode == 0) k_adjoint<0><<<grid, 256, 0, s>>>(a);
    else k_adjoint<1><<<grid, 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}
