/*
 * plain.cu — the plain path: neutron state as a structure of arrays in HBM
 * (lane l of neutron i at soa[l*stride + i]) and one kernel per reference
 * call site:
 *   k_generate      gen_prg (flat_mod.cl:4, cont_mod.cl:11)
 *   k_linear<S>     one component of a linear block: the reference's five
 *                   launches transform, intersect, terminate, scatter,
 *                   untransform (mcramp.py:124-157) fused into one pass
 *   k_nonlinear     one non-linear block, all its events (mcramp.py:167-217)
 * Each thread owns one neutron per grid-stride step; loads and stores of a
 * lane are contiguous across a warp (128-byte transactions).  Dead
 * neutrons cost one 4-byte read of the die lane; live ones read and write
 * only the lanes their component touches (the S template parameter fixes
 * that set at compile time).
 */
#include "device.cuh"
#include "launch.h"

#define PLAIN_BLOCK 256

#define LANES_APPLY(OP, n, S, st, i)                                                      \
  OP(n.x, RAMP_X) OP(n.y, RAMP_Y) OP(n.z, RAMP_Z) OP(n.vx, RAMP_VX) OP(n.vy, RAMP_VY)      \
  OP(n.vz, RAMP_VZ) OP(n.px, RAMP_PX) OP(n.py, RAMP_PY) OP(n.pz, RAMP_PZ) OP(n.p, RAMP_P) \
  OP(n.t, RAMP_TOF) OP(n.sb, RAMP_MC) OP(n.sc, RAMP_PREVCOMP) OP(n.sd, RAMP_SD)           \
  OP(n.se, RAMP_SE) OP(n.die, RAMP_DIE)
#define LD_(f, L) f = S[(L) * st + i];
#define ST_(f, L) S[(L) * st + i] = f;
#define LOAD_ALL(n, S, st, i) LANES_APPLY(LD_, n, S, st, i)
#define STORE_ALL(n, S, st, i) LANES_APPLY(ST_, n, S, st, i)
#define PLAIN_MAX_GRID (152 * 64)

/* scatter dispatch with the kind fixed at compile time when SK >= 0 */
template <int SK>
DI void scatter_k(const CompDev& c, Nt& n, Is& s, uint32_t& ii, Rng& r, StatusDev* st,
                  float* ev = nullptr) {
  if constexpr (SK == RAMP_S_RESCAL) {
    s_rescal(c, n, s, ii, r, ev);
    return;
  }
  switch (SK >= 0 ? SK : c.scat) {
    case RAMP_S_ARM: ii = c.idx; is_reset(s); break;
    case RAMP_S_GUIDE: s_guide(c, n, s, ii, st); break;
    case RAMP_S_CHOPPER: s_chopper(c, n, s, ii, r); break;
    case RAMP_S_ISOTROPIC: s_isotropic(c, n, s, ii, r); break;
    case RAMP_S_POWDERN: s_powdern(c, n, s, ii, r, st); break;
    case RAMP_S_DET1D: s_det1d(c, n, s, ii, st); break;
    case RAMP_S_DET2D: s_det2d(c, n, s, ii, st); break;
    case RAMP_S_COUNTER:
      if (c.tally) atomicAdd(c.tally, n.p);
      n.se = 1.0f; n.wr |= WR_SE;
      s_finish(c, n, s, ii);
      break;
    case RAMP_S_BEAMSTOP: set_die(n, 1.0f); s_finish(c, n, s, ii); break;
    case RAMP_S_ATTENUATE: s_attenuate(c, n, s, ii); break;
    case RAMP_S_MONO: s_mono(c, n, s, ii, r); break;
    case RAMP_S_POWDER1: s_powder1(c, n, s, ii, r); break;
    default: break;
  }
}

template <int SK, bool MESH>
DI void comp_linear_k(const CompDev& c, Nt& n, uint32_t& ii, Rng& r, StatusDev* st,
                      float* ev = nullptr) {
  transform(c, n);
  Is s;
  is_reset(s);
  if (intersect<MESH>(c, n, s, st)) ii = c.idx;
  if (len3(ip2(s)) == 0.0f && c.restore == 0) set_die(n, 1.f);
  if (ii == c.idx && !(n.die > 0.f)) scatter_k<SK>(c, n, s, ii, r, st, ev);
  if (!(n.die > 0.f)) untransform(c, n);
}

template <int MODE>
__global__ void __launch_bounds__(PLAIN_BLOCK)
k_generate(const __grid_constant__ SrcDev src, const PlainArgs a, int32_t num_sim, int32_t seed) {
  const int64_t st = a.stride;
  float* __restrict__ S = a.soa;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float old_sb = S[RAMP_MC * st + i];
    Nt n;
    Rng r;
    rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, 0u, a.rng.run_seed, a.rng.one);
    generate(src, n, old_sb, num_sim, a.rng.seed_dev ? *a.rng.seed_dev : seed, r);
    STORE_ALL(n, S, st, i);
  }
}

/* MESH: the component's geometry is a GMesh (only then is the hierarchy
 * walk compiled in: its stack raises register pressure in the whole kernel) */
template <int SK, int MODE, bool MESH>
__global__ void __launch_bounds__(PLAIN_BLOCK)
k_linear(const __grid_constant__ CompDev c, const PlainArgs a) {
  constexpr bool RD_P = SK == RAMP_S_GUIDE || SK == RAMP_S_ISOTROPIC || SK == RAMP_S_POWDERN ||
                        SK == RAMP_S_DET1D || SK == RAMP_S_DET2D || SK == RAMP_S_COUNTER ||
                        SK == RAMP_S_ATTENUATE || SK == RAMP_S_MONO || SK == RAMP_S_POWDER1 ||
                        SK == RAMP_S_RESCAL;
  constexpr bool RD_T = SK == RAMP_S_GUIDE || SK == RAMP_S_CHOPPER || SK == RAMP_S_ISOTROPIC ||
                        SK == RAMP_S_POWDERN || SK == RAMP_S_DET1D || SK == RAMP_S_DET2D ||
                        SK == RAMP_S_ATTENUATE || SK == RAMP_S_MONO || SK == RAMP_S_POWDER1;
  constexpr bool RD_SB = SK == RAMP_S_CHOPPER || SK == RAMP_S_ISOTROPIC || SK == RAMP_S_POWDERN ||
                         SK == RAMP_S_MONO || SK == RAMP_S_POWDER1 || SK == RAMP_S_RESCAL;
  constexpr bool MOD_VEL = SK == RAMP_S_GUIDE || SK == RAMP_S_ISOTROPIC || SK == RAMP_S_POWDERN ||
                           SK == RAMP_S_MONO || SK == RAMP_S_POWDER1 || SK == RAMP_S_RESCAL;
  constexpr bool USE_POL = SK == RAMP_S_ISOTROPIC;
  const int64_t st = a.stride;
  float* __restrict__ S = a.soa;
  const bool pol = USE_POL || c.rotated;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float die = S[RAMP_DIE * st + i];
    if (die > 0.f) continue;
    Nt n;
    n.wr = 0;
    n.die = die;
    n.x = S[RAMP_X * st + i];   n.y = S[RAMP_Y * st + i];   n.z = S[RAMP_Z * st + i];
    n.vx = S[RAMP_VX * st + i]; n.vy = S[RAMP_VY * st + i]; n.vz = S[RAMP_VZ * st + i];
    n.px = n.py = n.pz = 0.0f;
    if (pol) { n.px = S[RAMP_PX * st + i]; n.py = S[RAMP_PY * st + i]; n.pz = S[RAMP_PZ * st + i]; }
    n.p = RD_P ? S[RAMP_P * st + i] : 0.0f;
    n.t = RD_T ? S[RAMP_TOF * st + i] : 0.0f;
    n.sb = RD_SB ? S[RAMP_MC * st + i] : 0.0f;
    n.sc = n.sd = n.se = 0.0f;
    const uint32_t ii0 = a.iidx[i];
    uint32_t ii = ii0;
    Rng r;
    rng_init(r, MODE, a.rng.tid_base + (uint32_t)i, 0u, a.rng.run_seed, a.rng.one);
    float ev[8];
    comp_linear_k<SK, MESH>(c, n, ii, r, a.st, ev);
    if constexpr (SK == RAMP_S_RESCAL) {
      /* the event of a neutron this component scattered (rescal.cl:67) */
      if (n.wr & WR_SC) {
        if (c.tally && 8 * i + 8 <= c.tally_len) {
          float4* e = reinterpret_cast<float4*>(c.tally + 8 * i);
          e[0] = make_float4(ev[0], ev[1], ev[2], ev[3]);
          e[1] = make_float4(ev[4], ev[5], ev[6], ev[7]);
        } else {
          atomicAdd(&a.st->oob, 1ull);
        }
      }
    }
    S[RAMP_X * st + i] = n.x; S[RAMP_Y * st + i] = n.y; S[RAMP_Z * st + i] = n.z;
    if (MOD_VEL || c.rotated) {
      S[RAMP_VX * st + i] = n.vx; S[RAMP_VY * st + i] = n.vy; S[RAMP_VZ * st + i] = n.vz;
    }
    if (pol) { S[RAMP_PX * st + i] = n.px; S[RAMP_PY * st + i] = n.py; S[RAMP_PZ * st + i] = n.pz; }
    if (RD_P) S[RAMP_P * st + i] = n.p;
    if (RD_T) S[RAMP_TOF * st + i] = n.t;
    if (RD_SB) S[RAMP_MC * st + i] = n.sb;
    if (n.wr & WR_SC) S[RAMP_PREVCOMP * st + i] = n.sc;
    if (n.wr & WR_SD) S[RAMP_SD * st + i] = n.sd;
    if (n.wr & WR_SE) S[RAMP_SE * st + i] = n.se;
    if (n.wr & WR_DIE) S[RAMP_DIE * st + i] = n.die;
    if (ii != ii0) a.iidx[i] = ii;
  }
}

template <bool MESH>
__global__ void __launch_bounds__(PLAIN_BLOCK)
k_nonlinear(const CompDev* __restrict__ comps, int first, int count, int multi, const PlainArgs a) {
  const int64_t st = a.stride;
  float* __restrict__ S = a.soa;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float die = S[RAMP_DIE * st + i];
    if (die > 0.f) continue;
    Nt n;
    LOAD_ALL(n, S, st, i);
    n.wr = 0;
    uint32_t ii = a.iidx[i];
    Rng r;
    rng_init(r, a.rng.mode, a.rng.tid_base + (uint32_t)i, 0u, a.rng.run_seed, a.rng.one);
    block_nonlinear<NoDiff, true, MESH>(comps, first, count, multi, n, ii, r, a.st);
    STORE_ALL(n, S, st, i);
    a.iidx[i] = ii;
  }
}

static int plain_grid(int64_t n) {
  int64_t g = (n + PLAIN_BLOCK - 1) / PLAIN_BLOCK;
  if (g > PLAIN_MAX_GRID) g = PLAIN_MAX_GRID;
  if (g < 1) g = 1;
  return (int)g;
}

/* A host component (MCPL output or input, scatter done on the host)
 * splits its linear pass (mcramp.py:124-157) around the host action:
 * k_enter transforms into the component frame, intersects and terminates;
 * k_leave transforms back. */
__global__ void __launch_bounds__(PLAIN_BLOCK)
k_enter(const __grid_constant__ CompDev c, const PlainArgs a) {
  const int64_t st = a.stride;
  float* __restrict__ S = a.soa;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (S[RAMP_DIE * st + i] > 0.f) continue;
    Nt n;
    LOAD_ALL(n, S, st, i);
    n.wr = 0;
    uint32_t ii = a.iidx[i];
    transform(c, n);
    Is s;
    is_reset(s);
    if (intersect(c, n, s, a.st)) ii = c.idx;
    if (len3(ip2(s)) == 0.0f && c.restore == 0) set_die(n, 1.f);
    STORE_ALL(n, S, st, i);
    a.iidx[i] = ii;
  }
}

__global__ void __launch_bounds__(PLAIN_BLOCK)
k_leave(const __grid_constant__ CompDev c, const PlainArgs a) {
  const int64_t st = a.stride;
  float* __restrict__ S = a.soa;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (S[RAMP_DIE * st + i] > 0.f) continue;
    Nt n;
    LOAD_ALL(n, S, st, i);
    untransform(c, n);
    STORE_ALL(n, S, st, i);
  }
}

cudaError_t launch_host_half(const CompDev& c, const PlainArgs& a, int leave, cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.n <= 0) return cudaSuccess;
  if (leave) k_leave<<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(c, a);
  else k_enter<<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(c, a);
  return cudaGetLastError();
}

/* Order-preserving compaction of the records that are not dead (die lane
 * not exactly 1, the test of mcpl_out.py:103) into rows of the selected
 * lanes: per 1024-index tile a count, one scan of the tile counts, then
 * each record goes to its tile offset plus its rank inside the tile
 * (warp ballots).  The rows keep the index order. */
#define GATHER_TILE 1024

__global__ void __launch_bounds__(GATHER_TILE)
k_alive_count(const float* __restrict__ die, int64_t n, int64_t* __restrict__ tile_count) {
  __shared__ int warp_n[GATHER_TILE / 32];
  const int64_t i = (int64_t)blockIdx.x * GATHER_TILE + threadIdx.x;
  const bool keep = i < n && !(die[i] == 1.0f);
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < GATHER_TILE / 32; ++w) t += warp_n[w];
    tile_count[blockIdx.x] = t;
  }
}

/* exclusive scan of the tile counts in place (one CTA; each thread sums a
 * contiguous run, then the runs are scanned) and the total */
__global__ void __launch_bounds__(1024)
k_scan_tiles(int64_t* __restrict__ c, int64_t nt, int64_t* __restrict__ total) {
  __shared__ int64_t part[1024];
  const int64_t per = (nt + 1023) / 1024;
  const int64_t b = threadIdx.x * per, e = (b + per < nt) ? b + per : nt;
  int64_t sum = 0;
  for (int64_t k = b; k < e; ++k) sum += c[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int t = 0; t < 1024; ++t) { const int64_t v = part[t]; part[t] = run; run += v; }
    *total = run;
  }
  __syncthreads();
  int64_t run = part[threadIdx.x];
  for (int64_t k = b; k < e; ++k) { const int64_t v = c[k]; c[k] = run; run += v; }
}

__global__ void __launch_bounds__(GATHER_TILE)
k_alive_gather(const float* __restrict__ S, int64_t st, int64_t n,
               const int64_t* __restrict__ tile_off, uint32_t lanes, int nl,
               float* __restrict__ out) {
  __shared__ int warp_off[GATHER_TILE / 32];
  const int64_t i = (int64_t)blockIdx.x * GATHER_TILE + threadIdx.x;
  const bool keep = i < n && !(S[RAMP_DIE * st + i] == 1.0f);
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_off[w] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < GATHER_TILE / 32; ++k) { const int v = warp_off[k]; warp_off[k] = run; run += v; }
  }
  __syncthreads();
  if (!keep) return;
  const int64_t row = tile_off[blockIdx.x] + warp_off[w] + __popc(m & ((1u << lane) - 1u));
  float* o = out + row * nl;
  int k = 0;
  for (int l = 0; l < RAMP_NLANES; ++l)
    if (lanes & (1u << l)) o[k++] = S[(int64_t)l * st + i];
}

cudaError_t launch_gather_alive(const PlainArgs& a, uint32_t lanes, float* out, int64_t* scratch,
                                int64_t* total, cudaStream_t s) {
  const int64_t nt = (a.n + GATHER_TILE - 1) / GATHER_TILE;
  if (nt <= 0) return cudaMemsetAsync(total, 0, sizeof(int64_t), s);
  int nl = __builtin_popcount(lanes);
  k_alive_count<<<(unsigned)nt, GATHER_TILE, 0, s>>>(a.soa + (int64_t)RAMP_DIE * a.stride, a.n,
                                                     scratch);
  k_scan_tiles<<<1, 1024, 0, s>>>(scratch, nt, total);
  k_alive_gather<<<(unsigned)nt, GATHER_TILE, 0, s>>>(a.soa, a.stride, a.n, scratch, lanes, nl,
                                                      out);
  return cudaGetLastError();
}

cudaError_t launch_generate(const SrcDev& src, const PlainArgs& a, int32_t num_sim, int32_t seed,
                            cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.n <= 0) return cudaSuccess;
  if (a.rng.mode == 0) k_generate<0><<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(src, a, num_sim, seed);
  else k_generate<1><<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(src, a, num_sim, seed);
  return cudaGetLastError();
}

cudaError_t launch_linear_comp(const CompDev& c, const PlainArgs& a, cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.n <= 0) return cudaSuccess;
  int g = plain_grid(a.n);
  const bool mesh = c.geom == RAMP_G_MESH;
  switch (c.scat) {
/* kinds that draw random numbers get one instantiation per keying mode */
#define CASE(K)                                                               \
  case K:                                                                     \
    if (mesh) k_linear<K, 0, true><<<g, PLAIN_BLOCK, 0, s>>>(c, a);           \
    else k_linear<K, 0, false><<<g, PLAIN_BLOCK, 0, s>>>(c, a);               \
    break;
#define CASE2(K)                                                              \
  case K:                                                                     \
    if (mesh) {                                                               \
      if (a.rng.mode == 0) k_linear<K, 0, true><<<g, PLAIN_BLOCK, 0, s>>>(c, a); \
      else k_linear<K, 1, true><<<g, PLAIN_BLOCK, 0, s>>>(c, a);              \
    } else {                                                                  \
      if (a.rng.mode == 0) k_linear<K, 0, false><<<g, PLAIN_BLOCK, 0, s>>>(c, a); \
      else k_linear<K, 1, false><<<g, PLAIN_BLOCK, 0, s>>>(c, a);             \
    }                                                                         \
    break;
    CASE(RAMP_S_ARM) CASE(RAMP_S_GUIDE) CASE2(RAMP_S_CHOPPER) CASE2(RAMP_S_ISOTROPIC)
    CASE2(RAMP_S_POWDERN) CASE(RAMP_S_DET1D) CASE(RAMP_S_DET2D) CASE(RAMP_S_COUNTER)
    CASE(RAMP_S_BEAMSTOP) CASE(RAMP_S_ATTENUATE) CASE2(RAMP_S_MONO) CASE2(RAMP_S_POWDER1)
    CASE2(RAMP_S_RESCAL)
#undef CASE
#undef CASE2
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_nonlinear_block(const CompDev* comps_dev, int first, int count, int multi,
                                   bool mesh, const PlainArgs& a, cudaStream_t s) {
  if (a.rng.one != 1u) return cudaErrorInvalidValue;   /* tf20 */
  if (a.n <= 0 || multi <= 0 || count <= 0) return cudaSuccess;
  if (mesh) k_nonlinear<true><<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(comps_dev, first, count, multi, a);
  else k_nonlinear<false><<<plain_grid(a.n), PLAIN_BLOCK, 0, s>>>(comps_dev, first, count, multi, a);
  return cudaGetLastError();
}

/* ------------------------------------------------------------------ */
/* debug kernels used by the parity tests                               */
/* ------------------------------------------------------------------ */
__global__ void k_debug_threefry(const uint32_t* c0, const uint32_t* tid, uint32_t* out, int64_t n,
                                 uint32_t one) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t t = tid[i];
  out[i] = tf_ref_x(c0[i], t, TF_PARITY ^ t ^ TF_K1 ^ TF_K2 ^ TF_K3, one);
}

__global__ void k_debug_math(int fn, const float* a, const float* b, float* out, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = a[i], y = b ? b[i] : 0.0f, r = 0.0f;
  switch (fn) {
    case 0: r = rm_expf(x); break;
    case 1: r = rm_logf(x); break;
    case 2: r = rm_sinf(x); break;
    case 3: r = rm_cosf(x); break;
    case 4: r = rm_atan2f(x, y); break;
    case 5: r = rm_asinf(x); break;
    case 6: r = rm_acosf(x); break;
    case 7: r = rm_tanhf(x); break;
    case 8: r = rm_expm1f(x); break;
    case 9: r = reflectivity(x, 0.99f, 0.0219f, 3.0f, 2.0f, 0.003f); break;
    default: break;
  }
  out[i] = r;
}

__global__ void __launch_bounds__(256) k_debug_rng_peak(int32_t iters, uint32_t* out, int64_t n,
                                                        uint32_t one) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t tid = (uint32_t)i;
  uint32_t k4 = TF_PARITY ^ tid ^ TF_K1 ^ TF_K2 ^ TF_K3;
  uint32_t a = tid, b = tid ^ 0x9e3779b9u;
  for (int k = 0; k < iters; ++k) {
    a = tf_ref_x(a, tid, k4, one);
    b = tf_ref_x(b, tid, k4, one);
  }
  out[i] = a ^ b;
}

cudaError_t launch_debug_rng_peak(int64_t n, int32_t iters, uint32_t* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_debug_rng_peak<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(iters, out, n, 1u);
  return cudaGetLastError();
}

/* L2 read bandwidth: every thread reads `iters` float4 of a buffer of len
 * float4 (a power of two, small enough to stay in L2) through loads that
 * bypass L1 (ld.global.cg); the warps of a pass read consecutive 512-byte
 * runs.  out[thread] keeps the sums live. */
__global__ void __launch_bounds__(256) k_debug_l2_peak(const float4* __restrict__ buf,
                                                        uint64_t mask, int32_t iters,
                                                        float* out) {
  const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t j = i;
  float a0 = 0.0f, a1 = 0.0f;
  for (int k = 0; k < iters; k += 2) {
    const float4 u = __ldcg(buf + (j & mask));
    const float4 v = __ldcg(buf + ((j + nt) & mask));
    a0 += (u.x + u.y) + (u.z + u.w);
    a1 += (v.x + v.y) + (v.z + v.w);
    j += 2 * nt;
  }
  out[i] = a0 + a1;
}

cudaError_t launch_debug_l2_peak(const float4* buf, int64_t len4, int64_t n, int32_t iters,
                                 float* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_debug_l2_peak<<<(unsigned)(n / 256), 256, 0, s>>>(buf, (uint64_t)len4 - 1, iters, out);
  return cudaGetLastError();
}

/* L2 float-atomic throughput: every thread adds 1 to `iters` bins of an
 * L2-resident histogram of n_bins floats (a power of two), the 32 lanes of
 * a warp to 32 consecutive bins (one 128-byte line), no two lanes of a
 * warp on one bin, as the tallies' warp-aggregated adds issue them. */
__global__ void __launch_bounds__(256) k_debug_atomic_peak(float* bins, uint32_t mask,
                                                            int32_t iters) {
  const uint32_t nt = gridDim.x * blockDim.x;
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  for (int k = 0; k < iters; ++k) {
    atomicAdd(bins + (j & mask), 1.0f);
    j += nt;
  }
}

cudaError_t launch_debug_atomic_peak(float* bins, int64_t n_bins, int64_t n, int32_t iters,
                                     cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_debug_atomic_peak<<<(unsigned)(n / 256), 256, 0, s>>>(bins, (uint32_t)(n_bins - 1), iters);
  return cudaGetLastError();
}

/* next chunk seed in [0, 4096] from a 64-bit LCG (Knuth's MMIX constants) */
__global__ void k_seed_advance(int32_t* seed_dev) {
  unsigned long long* st = reinterpret_cast<unsigned long long*>(seed_dev + 2);
  unsigned long long x = *st * 6364136223846793005ull + 1442695040888963407ull;
  *st = x;
  seed_dev[0] = (int32_t)((x >> 33) % 4097ull);
}

cudaError_t launch_seed_advance(int32_t* seed_dev, cudaStream_t s) {
  k_seed_advance<<<1, 1, 0, s>>>(seed_dev);
  return cudaGetLastError();
}

cudaError_t launch_debug_threefry(const uint32_t* c0, const uint32_t* tid, uint32_t* out,
                                  int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_debug_threefry<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c0, tid, out, n, 1u);
  return cudaGetLastError();
}

cudaError_t launch_debug_math(int fn, const float* a, const float* b, float* out, int64_t n,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_debug_math<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fn, a, b, out, n);
  return cudaGetLastError();
}
