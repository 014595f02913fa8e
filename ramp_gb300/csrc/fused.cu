/*
 * fused.cu — dispatch of the fused persistent kernel (fused_kernel.cuh)
 * over its register caps, keying modes, layouts and kind sets, and the
 * sequencing of a split launch (stage A, then stage B).  The kernels are
 * instantiated one per translation unit (fused_inst.cu).
 */
#include "fused_kernel.cuh"

#define PH(MB, MODE, B, PHASE, KS)                                                          \
  extern template cudaError_t launch_phase<MB, MODE, B, PHASE, KS>(const FusedArgs&, int, int, \
                                                                   cudaStream_t);
/* kind sets: 0 the core kinds, 1 everything (extended kinds: MISIS source,
   SMonochromator, SPowder1, and the mesh), 2 the core kinds and the mesh */
#define ONE_MODE(MB, MODE)                                                                  \
  PH(MB, MODE, false, 0, 0) PH(MB, MODE, false, 1, 0) PH(MB, MODE, false, 2, 0)             \
  PH(MB, MODE, true, 0, 0) PH(MB, MODE, true, 1, 0) PH(MB, MODE, true, 2, 0)                \
  PH(MB, MODE, false, 0, 1) PH(MB, MODE, false, 1, 1) PH(MB, MODE, false, 2, 1)             \
  PH(MB, MODE, true, 0, 1)                                                                  \
  PH(MB, MODE, false, 0, 2) PH(MB, MODE, false, 1, 2) PH(MB, MODE, false, 2, 2)             \
  PH(MB, MODE, true, 0, 2) PH(MB, MODE, true, 1, 2) PH(MB, MODE, true, 2, 2)                \
  PH(MB, MODE, false, 4, 2) PH(MB, MODE, true, 4, 2)                                        \
  PH(MB, MODE, false, 5, 2) PH(MB, MODE, true, 5, 2)                                        \
  PH(MB, MODE, false, 3, 0) PH(MB, MODE, true, 3, 0)                                        \
  extern template int occ_mm<MB, MODE>(int);
ONE_MODE(3, 0)
ONE_MODE(3, 1)
ONE_MODE(4, 0)
ONE_MODE(4, 1)

/* ---- before the lean stage A: the speed look-ahead -------------------
 * The speed table of a variant (lookahead.h: the run's constants, ordered,
 * and a verdict for each cell of 1 / speed) lives in word 19 of the
 * variant's survivor slots, free on this path; a variant without the speed
 * look-ahead, or with fewer slots than the table takes, has none. */
template <bool BATCHED>
DI uint32_t* speed_tab_slot(const FusedArgs& a, const VariantDev* V) {
  const int64_t n = V->n;
  const int64_t item0 = BATCHED ? V->item_off : 0;
  const int64_t items = (n + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK;
  const bool speed = (V->src.kind == RAMP_SRC_FLAT || V->src.kind == RAMP_SRC_CONT) &&
                     a.carry_sb == nullptr && a.cull > 0;
  if (!speed || item0 + items > a.surv_items || items * FUSED_WARP_TASK < SPEED_TAB_WORDS)
    return nullptr;
  return a.surv + (size_t)19 * a.surv_cap + item0 * FUSED_WARP_TASK;
}

/* the speed table of each variant: one grid row per variant, SPEED_CELLS /
 * 256 CTAs of 256 threads a row, each CTA preparing and ordering the run
 * and deciding 256 cells; CTA 0 also writes the run and the cell layout.
 * The cells cover 1 / speed of the moderator's energy range (flat_mod.cl,
 * cont_mod.cl:36: v = SE2V sqrt(E), E uniform in [E_min, E_max]) widened
 * by 1e-5 of it; a history outside them takes speed_run_blocks. */
template <bool BATCHED>
__global__ void __launch_bounds__(256) k_speed_table(const FusedArgs a) {
  const int var = BATCHED ? (int)blockIdx.y : a.var_key;
  const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
  uint32_t* const dst = speed_tab_slot<BATCHED>(a, V);
  if (dst == nullptr) return;
  __shared__ SpeedTab T;
  __shared__ int blocked[SPEED_RUN_MAX];
  speed_tab_build(dst, &T, blocked, V->comps, a.cull, V->src.p, (int)blockIdx.x);
}

/* the keep pass over histories [0, n) of one variant (index type I: 32-bit
 * when the grid's strides stay below 2^31); `test` false lists every one */
template <typename I, int MODE>
DI void keep_histories(const FusedArgs& a, const SrcDev& src, const SpeedTab& tab, bool test,
                       int var, int32_t seed, I n, uint32_t* keep, unsigned long long* kc,
                       uint32_t* stage) {
  const int lane = threadIdx.x & 31;
  int held = 0;
  const I stride = (I)gridDim.x * (I)blockDim.x;
  for (I base = (I)blockIdx.x * (I)blockDim.x + (I)(threadIdx.x & ~31); base < n;
       base += stride) {                                   /* warp-uniform */
    const I i = base + (I)lane;
    bool kept = false;
    if (i < n) {
      kept = true;
      if (test) {
        /* generate's first draw and speed (flat_mod.cl, cont_mod.cl:36) */
        Rng r;
        rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, (uint32_t)var, a.rng.run_seed,
                 a.rng.one);
        Nt nn;
        nn.sb = (float)seed + 0.0f;
        kept = !speed_tab_blocks(tab, draw_word(nn, r));
      }
    }
    warp_list_add(kept, (uint32_t)i, stage, held, kc, keep, (int64_t)n);
  }
  warp_list_flush(stage, held, kc, keep, (int64_t)n);
}

/* Every history's first draw (its energy, hence its speed) is made here
 * and the speed-only bound applied (speed_tab_blocks on the draw's word,
 * with the variant's speed table; without one, speed_run_blocks with the
 * run prepared here);
 * the indices of the histories that may pass are appended (warp_list_add)
 * to a list in word 18 of the variant's survivor slots (free until a walk
 * uses it), its length in the variant's workq_c.  The lean stage A then
 * traces only the listed histories, each regenerated from its key (the
 * same operations, so the same neutron).  Without carry buffers only; with
 * a source other than flat or MCont every history is listed. */
template <int MODE, bool BATCHED>
__global__ void __launch_bounds__(256) k_speed_keep(const FusedArgs a) {
  const int var = BATCHED ? (int)blockIdx.y : a.var_key;
  const VariantDev* __restrict__ V = BATCHED ? a.variants + var : &a.single;
  const int64_t n = V->n;
  const int64_t item0 = BATCHED ? V->item_off : 0;
  if (BATCHED && item0 + (n + FUSED_WARP_TASK - 1) / FUSED_WARP_TASK > a.surv_items) return;
  const SrcDev& src = V->src;
  const bool speed = (src.kind == RAMP_SRC_FLAT || src.kind == RAMP_SRC_CONT) &&
                     a.carry_sb == nullptr && a.cull > 0;
  uint32_t* const keep = a.surv + (size_t)18 * a.surv_cap + item0 * FUSED_WARP_TASK;
  unsigned long long* const kc = a.workq_c + (BATCHED ? var : 0);
  const int32_t seed = (a.rng.seed_dev && !BATCHED) ? *a.rng.seed_dev : V->seed;
  /* the variant's speed table, or the run prepared here without cells */
  __shared__ SpeedTab tab;
  const uint32_t* const tsrc = speed_tab_slot<BATCHED>(a, V);
  if (tsrc != nullptr) {
    speed_tab_load(&tab, tsrc);
  } else {
    __shared__ int blocked[SPEED_RUN_MAX];
    speed_run_setup(&tab.run, blocked, speed, V->comps, a.cull, src.p);
    if (threadIdx.x == 0) {
      speed_tab_range(&tab, src.p[5], src.p[6] - src.p[5]);
      tab.ncell = 0;                 /* no cells: every history takes the run */
    }
    __syncthreads();
  }
  __shared__ uint32_t stage[256 / 32][64];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const bool test = speed && tab.run.n > 0;
  if (n + stride <= (int64_t)INT32_MAX)
    keep_histories<int32_t, MODE>(a, src, tab, test, var, seed, (int32_t)n, keep, kc,
                                  stage[threadIdx.x >> 5]);
  else
    keep_histories<int64_t, MODE>(a, src, tab, test, var, seed, n, keep, kc,
                                  stage[threadIdx.x >> 5]);
}

/* one register cap, keying mode, layout and kind set: the whole chain, or
 * stage A then stage B of a split launch (the batched one-launch layout
 * runs the extended kinds whole; the mesh walk runs with the mesh kind set;
 * a split before component 0 of a core-kind chain, which only the chopper
 * look-ahead makes, has a stage A of its own without the component code) */
template <int MB, int MODE, bool BATCHED, int KS>
static cudaError_t launch_fk(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if constexpr (KS == 2) {
    if (a.walk) {      /* stage A, the walk, then the rest of the chain */
      cudaError_t e = launch_phase<MB, MODE, BATCHED, 1, 2>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      e = launch_phase<MB, MODE, BATCHED, 4, 2>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 5, 2>(a, block, grid, s);
    }
  }
  if constexpr (!(BATCHED && KS == 1)) {
    if (a.split > 0 || a.cull > 0) {
      cudaError_t e;
      if (KS == 0 && a.split == 0) {   /* the moderator alone: the lean stage A */
        const unsigned rows = BATCHED ? (unsigned)a.n_variants : 1u;
        k_speed_table<BATCHED><<<dim3(SPEED_CELLS / 256, rows), 256, 0, s>>>(a);
        k_speed_keep<MODE, BATCHED><<<dim3((unsigned)grid, rows), 256, 0, s>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = launch_phase<MB, MODE, BATCHED, 3, 0>(a, block, grid, s);
      } else
        e = launch_phase<MB, MODE, BATCHED, 1, KS>(a, block, grid, s);
      if (e != cudaSuccess) return e;
      return launch_phase<MB, MODE, BATCHED, 2, KS>(a, block, grid, s);
    }
  }
  return launch_phase<MB, MODE, BATCHED, 0, KS>(a, block, grid, s);
}

template <int MB, int MODE>
static cudaError_t launch_m(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  switch (a.ext) {
    case 1:
      return a.variants ? launch_fk<MB, MODE, true, 1>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 1>(a, block, grid, s);
    case 2:
      return a.variants ? launch_fk<MB, MODE, true, 2>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 2>(a, block, grid, s);
    default:
      return a.variants ? launch_fk<MB, MODE, true, 0>(a, block, grid, s)
                        : launch_fk<MB, MODE, false, 0>(a, block, grid, s);
  }
}

cudaError_t launch_fused(const FusedArgs& a, int block, int grid, cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.variants ? a.n_variants <= 0 : a.n_tasks <= 0) return cudaSuccess;
  if (a.variants && a.n_variants > 65535) return cudaErrorInvalidValue;   /* grid rows */
  if (a.n_blocks > FUSED_MAX_BLOCKS || a.n_comps > RAMP_MAX_COMPS) return cudaErrorInvalidValue;
  if (a.split < 0 || ((a.split > 0 || a.cull > 0) && (a.split >= a.n_comps || !a.surv)))
    return cudaErrorInvalidValue;
  if (a.cull > 0 && (a.walk || a.split + a.cull > a.n_comps || (a.variants && a.ext == 1)))
    return cudaErrorInvalidValue;
  if (a.walk && (a.ext != 2 || a.split >= a.n_comps || !a.surv || !a.workq_c))
    return cudaErrorInvalidValue;
  /* register cap: 3 or 4 CTAs of 256 threads per SM (at 2 the kernel is
     never faster on GB300) */
  if (a.minb != 3)
    return a.rng.mode == 0 ? launch_m<4, 0>(a, block, grid, s) : launch_m<4, 1>(a, block, grid, s);
  return a.rng.mode == 0 ? launch_m<3, 0>(a, block, grid, s) : launch_m<3, 1>(a, block, grid, s);
}

int fused_max_blocks_per_sm(int block, int minb) {
  return minb != 3 ? occ_mm<4, 0>(block) : occ_mm<3, 0>(block);
}
