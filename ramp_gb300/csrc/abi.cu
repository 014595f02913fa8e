/*
 * abi.cu — host side of the C ABI declared in include/ramp.h: plan
 * creation (descriptor validation, frame matrices, table and BVH upload),
 * the plain and fused launchers, status readback and error messages.
 */
#include <memory>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ramp.h"
#include "rmath.h"
#include "rconst.h"
#include "plan.h"
#include "launch.h"
#include "lookahead.h"
#include "bvh.h"

static thread_local std::string g_err;

static void set_err(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      set_err("%s: %s", #x, cudaGetErrorString(e_));                          \
      return e_ == cudaErrorMemoryAllocation ? RAMP_E_NOMEM : RAMP_E_CUDA;    \
    }                                                                         \
  } while (0)

struct BatchCache {
  std::vector<CompDev> comps_host;   /* n_variants * n_comps              */
  CompDev* comps_dev = nullptr;
  size_t comps_cap = 0;
  VariantDev* vars_dev = nullptr;
  size_t vars_cap = 0;
  std::vector<VariantDev> vars_host;
  unsigned long long* counters = nullptr;   /* per-variant work queues */
  size_t counters_cap = 0;
};

/* streams of the concurrent per-variant launches of ramp_trace_batched */
#define RAMP_BATCH_STREAMS 16
struct StreamSet {
  bool ready = false;
  int device = -1;
  cudaStream_t st[RAMP_BATCH_STREAMS];
  cudaEvent_t fork;
  cudaEvent_t join[RAMP_BATCH_STREAMS];
};

/* device copies of host tables, keyed by (kind, length, content hash) so
 * variants that share a table share one upload (kind 0 table, 1 BVH) */
typedef std::tuple<int, int64_t, uint64_t> TabKey;

/* what a recorded index list was made for (ramp_forward_record) */
struct RecKey {
  int64_t n;
  int32_t det, num_sim, seed, mode;
  uint32_t run_seed, tid_base;
  uint64_t version;
};

struct RampPlan {
  RampSource src_in;
  SrcDev src;
  std::vector<RampComp> comps_in;    /* the caller's descriptors           */
  std::vector<CompDev> comps;        /* host copy of device descriptors    */
  CompDev* comps_dev = nullptr;
  std::vector<RampBlock> blocks;
  RampBlock* blocks_dev = nullptr;
  StatusDev* status = nullptr;
  std::vector<std::pair<void*, size_t>> allocs;   /* small buffers (plan_alloc) */
  int sm_count = 0;
  int device = 0;                    /* the device the plan's buffers live on */
  BatchCache batch;
  std::map<TabKey, std::pair<void*, void*>> tabs;
  std::vector<CompDev> adj_host;     /* descriptors of the last adjoint   */
  CompDev* adj_dev = nullptr;
  uint32_t* adj_list = nullptr;      /* indices counted by the loss detector, */
  int64_t adj_cap = 0;               /* then its count (uint64) after them    */
  RecKey rec;                        /* the launch that filled adj_list       */
  bool rec_valid = false;
  uint64_t param_version = 0;        /* bumped when ramp_plan_set_param changes a value */
  CompDev* priv_dev = nullptr;       /* descriptors of a private-tally launch */
  uint32_t* surv = nullptr;          /* survivor buffer of split launches */
  int64_t surv_cap = 0;              /* slots (128 per work item) */
  bool surv_owned = false;           /* surv was allocated by the plan */
  uint32_t* surv_ext = nullptr;      /* caller's buffer (ramp_plan_set_survivors) */
  int64_t surv_ext_bytes = 0;
  StreamSet streams;
  bool plain_only = false;           /* a component writes per-index output */
  bool ext = false;                  /* an extended kind: MISIS, SMonochromator, SPowder1 */
  bool mesh = false;                 /* a GMesh or SAttenuate component */
};

static bool ext_source(const RampSource& s) { return s.kind == RAMP_SRC_ISIS; }

/* kind set of the whole-chain kernels a launch runs (FusedArgs.ext): the
 * extended kinds (with everything else) before the mesh, the mesh before
 * the core kinds alone */
static int32_t kind_set(bool ext, bool mesh) { return ext ? 1 : (mesh ? 2 : 0); }

/* whole-chain kernels (fused, batched, adjoint) cannot write per-index
 * component output */
static int check_whole_chain(const RampPlan* p, const char* who) {
  if (p->plain_only) {
    set_err("%s: the chain has a component that needs the plain path (SRescal events, "
            "host components)", who);
    return RAMP_E_UNSUPPORTED;
  }
  return RAMP_OK;
}

/* ---------------------------------------------------------------------- */
/* host float helpers: the same operations the device uses                 */
/* ---------------------------------------------------------------------- */
/* frame matrix, mcramp/include/geom.h:21-53 */
static void rot_matrix(const float* rot, float* R) {
  float x_a = rot[0], y_a = rot[1], z_a = rot[2];
  float cx = rm_cosf(x_a), sx = rm_sinf(x_a);
  float cy = rm_cosf(y_a), sy = rm_sinf(y_a);
  float cz = rm_cosf(z_a), sz = rm_sinf(z_a);
  R[0] = cy * cz;
  R[1] = -cx * sz + sx * sy * cz;
  R[2] = sx * sz + cx * sy * cz;
  R[3] = cy * sz;
  R[4] = cx * cz + sx * sy * sz;
  R[5] = -sx * cz + cx * sy * sz;
  R[6] = -sy;
  R[7] = sx * cy;
  R[8] = cx * cy;
}

/* maxwell_energy_distn, cont_mod.cl:4-9 */
static float maxwell_h(float E, float T) {
  float rootE = sqrtf(E);
  float overKT = 1.0f / (RC_K_B * T);
  return 2.0f * rootE / sqrtf(RC_PI) * (overKT * sqrtf(overKT)) * rm_expf(-E * overKT);
}

/* Guide constants that guide.cl:39-43 and ref.h:7-31 recompute for every
 * neutron and bounce, evaluated once with the same float operations:
 * aux[0] ww, [1] hh, [2] (-whalf)*l, [3] (-hhalf)*l, [4] l*l + ww*ww,
 * [5] sqrt of [4], [6] l*l + hh*hh, [7] sqrt of [6]; reflectivity after the
 * m-parametrisation: [8] m, [9] W, [10] alpha, [11] beta, [12] m*Qc,
 * [13] Qc after the m < 1 rescaling, [14] R0*0.5, [15] 1 if R = 0 always. */
static void guide_aux(const RampComp& c, float* aux) {
  const float w1 = c.sp[0], h1 = c.sp[1], w2 = c.sp[2], h2 = c.sp[3], l = c.sp[4];
  const float R0 = c.sp[5], Qc = c.sp[6];
  float alpha = c.sp[7], m = c.sp[8], W = c.sp[9];
  float ww = 0.5f * (w2 - w1), hh = 0.5f * (h2 - h1);
  float whalf = 0.5f * w1, hhalf = 0.5f * h1;
  aux[0] = ww;
  aux[1] = hh;
  aux[2] = -whalf * l;
  aux[3] = -hhalf * l;
  aux[4] = l * l + ww * ww;
  aux[5] = sqrtf(aux[4]);
  aux[6] = l * l + hh * hh;
  aux[7] = sqrtf(aux[6]);
  float beta = 0.0f;
  if (W == 0.0f && alpha == 0.0f) {
    m = m * 0.9853f + 0.1978f;
    W = -0.0002f * m + 0.0022f;
    alpha = 0.2304f * m + 5.0944f;
    beta = -7.6251f * m + 68.1137f;
    if (m <= 3) { alpha = m; beta = 0; }
  }
  aux[8] = m;
  aux[9] = W;
  aux[10] = alpha;
  aux[11] = beta;
  aux[12] = m * Qc;
  aux[13] = (m < 1) ? Qc * m : Qc;
  aux[14] = R0 * 0.5f;
  aux[15] = (m <= 0 || Qc <= 0 || R0 <= 0) ? 1.0f : 0.0f;
}

/* Device memory of plans' small buffers (descriptors, tables, status),
 * kept by size in a per-process pool once their plan is destroyed and
 * handed to the next plan: an Instrument built per run would otherwise
 * pay a cudaMalloc and a cudaFree per buffer.  ramp_plan_destroy waits
 * for the device before it returns buffers here, as cudaFree would, so
 * no kernel still reads one when it is reused.  At most 64 MB is kept. */
static std::mutex g_pool_mu;
static std::multimap<std::pair<int, size_t>, void*> g_pool;   /* (device, bytes) */
static size_t g_pool_bytes = 0;
static const size_t POOL_MAX = (size_t)64 << 20;

static size_t pool_round(size_t bytes) { return ((bytes > 0 ? bytes : 16) + 255) & ~(size_t)255; }

/* on the current device */
static cudaError_t plan_alloc(size_t bytes, void** dev,
                              std::vector<std::pair<void*, size_t>>& owner) {
  const size_t b = pool_round(bytes);
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pool.find(std::make_pair(d, b));
    if (it != g_pool.end()) {
      *dev = it->second;
      g_pool.erase(it);
      g_pool_bytes -= b;
      owner.push_back(std::make_pair(*dev, b));
      return cudaSuccess;
    }
  }
  e = cudaMalloc(dev, b);
  if (e == cudaSuccess) owner.push_back(std::make_pair(*dev, b));
  return e;
}

/* the buffers of a plan on device d, no longer read by any kernel */
static void plan_release(int d, std::vector<std::pair<void*, size_t>>& owner) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (auto& a : owner) {
    if (g_pool_bytes + a.second <= POOL_MAX) {
      g_pool.insert(std::make_pair(std::make_pair(d, a.second), a.first));
      g_pool_bytes += a.second;
    } else {
      cudaFree(a.first);
    }
  }
  owner.clear();
}

static int upload(const void* host, size_t bytes, void** dev,
                  std::vector<std::pair<void*, size_t>>& owner) {
  void* p = nullptr;
  CK(plan_alloc(bytes, &p, owner));
  if (bytes) CK(cudaMemcpy(p, host, bytes, cudaMemcpyHostToDevice));
  *dev = p;
  return RAMP_OK;
}

static int validate_comp(const RampComp& c, int j) {
  if (c.geom < RAMP_G_PLANE || c.geom > RAMP_G_MESH) {
    set_err("component %d: unknown geometry kind %d", j, c.geom);
    return RAMP_E_UNSUPPORTED;
  }
  if (c.scat < RAMP_S_ARM || c.scat > RAMP_S_HOST) {
    set_err("component %d: unknown scatter kind %d", j, c.scat);
    return RAMP_E_UNSUPPORTED;
  }
  if (c.geom == RAMP_G_PLANE && c.gi[0] != 0 && c.gi[0] != 1) {
    set_err("component %d: plane orientation %d", j, c.gi[0]);
    return RAMP_E_INVALID;
  }
  if (c.geom == RAMP_G_MESH && (c.table_len[0] <= 0 || c.table_len[0] % 9 || !c.table[0])) {
    set_err("component %d: mesh needs 9*n_tri points", j);
    return RAMP_E_INVALID;
  }
  if (c.scat == RAMP_S_ATTENUATE && c.geom != RAMP_G_MESH) {
    set_err("component %d: SAttenuate needs a GMesh geometry", j);
    return RAMP_E_INVALID;
  }
  if (c.scat == RAMP_S_POWDERN &&
      (c.si[0] < 1 || c.table_len[0] < c.si[0] || c.table_len[1] < c.si[0])) {
    set_err("component %d: powder line tables shorter than num_lines", j);
    return RAMP_E_INVALID;
  }
  if (c.scat == RAMP_S_ISOTROPIC) {
    for (int ch = 0; ch < 3; ++ch) {
      int64_t nq = c.si[1 + 2 * ch], nw = c.si[2 + 2 * ch];
      if (nq < 0 || nw < 0 || c.table_len[4 * ch] < nq || c.table_len[4 * ch + 1] < nw ||
          c.table_len[4 * ch + 2] < nw || c.table_len[4 * ch + 3] < nq * nw) {
        set_err("component %d: isotropic channel %d tables inconsistent", j, ch);
        return RAMP_E_INVALID;
      }
    }
  }
  if (c.scat == RAMP_S_DET1D && (c.si[2] != c.tally_len || !c.tally || !c.tally_err)) {
    set_err("component %d: 1-D detector tally length %lld != bins %d", j,
            (long long)c.tally_len, c.si[2]);
    return RAMP_E_INVALID;
  }
  if (c.scat == RAMP_S_DET2D &&
      ((int64_t)c.si[2] * c.si[3] != c.tally_len || !c.tally || !c.tally_err)) {
    set_err("component %d: 2-D detector tally length mismatch", j);
    return RAMP_E_INVALID;
  }
  return RAMP_OK;
}

static uint64_t fnv1a(const void* data, size_t bytes) {
  const unsigned char* b = (const unsigned char*)data;
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < bytes; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

/* content hash of a host table; within one call a table met again at the
 * same address is not re-hashed (memo, optional) */
typedef std::map<std::pair<const void*, int64_t>, uint64_t> HashMemo;
static uint64_t table_hash(const void* host, int64_t bytes, HashMemo* memo) {
  if (memo) {
    auto it = memo->find(std::make_pair(host, bytes));
    if (it != memo->end()) return it->second;
  }
  uint64_t h = fnv1a(host, (size_t)bytes);
  if (memo) (*memo)[std::make_pair(host, bytes)] = h;
  return h;
}

static int get_table(RampPlan* p, const float* host, int64_t len, const float** dev,
                     HashMemo* memo = nullptr) {
  static const float zero = 0.0f;
  if (len <= 0 || !host) { host = &zero; len = 1; }
  TabKey key(0, len, table_hash(host, len * (int64_t)sizeof(float), memo));
  auto it = p->tabs.find(key);
  if (it != p->tabs.end()) { *dev = (const float*)it->second.first; return RAMP_OK; }
  void* d;
  int rc = upload(host, (size_t)len * sizeof(float), &d, p->allocs);
  if (rc) return rc;
  p->tabs[key] = std::make_pair(d, (void*)nullptr);
  *dev = (const float*)d;
  return RAMP_OK;
}

static int lookup_table(RampPlan* p, const float* host, int64_t len, const float** dev,
                        HashMemo* memo);
static int lookup_bvh(RampPlan* p, const float* pts, int64_t len, const float4** nodes_dev,
                      const float4** tris_dev, HashMemo* memo);

/* device source descriptor; MISIS tables are uploaded (or, for callers
 * that may not allocate, looked up among the plan's tables) */
static int make_src(RampPlan* p, const RampSource& s, SrcDev& d, bool may_upload = true,
                    HashMemo* memo = nullptr) {
  if (s.kind != RAMP_SRC_FLAT && s.kind != RAMP_SRC_CONT && s.kind != RAMP_SRC_ISIS) {
    set_err("unknown source kind %d", s.kind);
    return RAMP_E_UNSUPPORTED;
  }
  memset(&d, 0, sizeof(d));
  d.kind = s.kind;
  d.dslot_T = -1;
  memcpy(d.p, s.p, sizeof(d.p));
  if (s.kind == RAMP_SRC_CONT) {
    d.dmax[0] = maxwell_h(RC_K_B * s.p[7], s.p[7]);
    d.dmax[1] = maxwell_h(RC_K_B * s.p[9], s.p[9]);
    d.dmax[2] = maxwell_h(RC_K_B * s.p[11], s.p[11]);
    for (int q = 0; q < 3; ++q) {          /* the per-neutron constants of M(E; T_q) */
      const float overKT = 1.0f / (RC_K_B * s.p[7 + 2 * q]);
      d.okt[q] = overKT;
      d.okc[q] = overKT * sqrtf(overKT);
    }
    /* I_q * M(E; T_q) / dmax_q is +0 for every drawn E >= 0 when I_q = 0
       and T_q, dmax_q are finite and positive: adding it changes no sum */
    const bool e_ok = s.p[5] >= 0.0f && s.p[6] >= 0.0f && std::isfinite(s.p[5]) &&
                      std::isfinite(s.p[6]);
    for (int q = 1; q < 3; ++q) {
      const float I = s.p[8 + 2 * q], T = s.p[7 + 2 * q], dm = d.dmax[q];
      if (e_ok && I == 0.0f && T > 0.0f && std::isfinite(T) && dm > 0.0f && std::isfinite(dm))
        d.zero_terms |= 1u << q;
    }
  }
  if (s.kind == RAMP_SRC_ISIS) {
    const int64_t nt = s.table_len[1], ne = s.table_len[2];
    if (nt < 2 || ne < 2 || s.table_len[0] != (ne - 1) * nt || s.table_len[3] != ne ||
        !s.table[0] || !s.table[1] || !s.table[2] || !s.table[3] || nt * ne > INT32_MAX) {
      set_err("MISIS: tables must hold (n_e-1)*n_t flux values, n_t times, n_e energies and "
              "n_e cumulative values, n_t, n_e >= 2");
      return RAMP_E_INVALID;
    }
    /* the device searches the two cumulative tables by bisection, which
       equals the reference's linear scan on non-decreasing tables */
    for (int k : {0, 3})
      for (int64_t i = 1; i < s.table_len[k]; ++i)
        if (!(s.table[k][i] >= s.table[k][i - 1])) {
          set_err("MISIS: cumulative table %d decreases at %lld", k, (long long)i);
          return RAMP_E_INVALID;
        }
    for (int k = 0; k < 4; ++k) {
      int rc = may_upload ? get_table(p, s.table[k], s.table_len[k], &d.tab[k], memo)
                          : lookup_table(p, s.table[k], s.table_len[k], &d.tab[k], memo);
      if (rc) {
        if (!may_upload) set_err("MISIS tables are not in the plan");
        return rc;
      }
    }
    d.n_t = (int32_t)nt;
    d.n_e = (int32_t)ne;
  }
  return RAMP_OK;
}

static int get_bvh(RampPlan* p, const float* pts, int64_t len, const float4** nodes_dev,
                   const float4** tris_dev, HashMemo* memo = nullptr) {
  TabKey key(1, len, table_hash(pts, len * (int64_t)sizeof(float), memo));
  auto it = p->tabs.find(key);
  if (it == p->tabs.end()) {
    std::vector<float> nodes, tris;
    if (ramp_bvh_build(pts, len / 9, nodes, tris) != 0) {
      set_err("BVH build failed");
      return RAMP_E_INVALID;
    }
    void *pn, *pt;
    int rc = upload(nodes.data(), nodes.size() * sizeof(float), &pn, p->allocs);
    if (rc) return rc;
    rc = upload(tris.data(), tris.size() * sizeof(float), &pt, p->allocs);
    if (rc) return rc;
    it = p->tabs.emplace(key, std::make_pair(pn, pt)).first;
  }
  *nodes_dev = (const float4*)it->second.first;
  *tris_dev = (const float4*)it->second.second;
  return RAMP_OK;
}

/* chopper constants: aux[0] the slit period 2 pi / n_slits (chopper.cl:21),
 * aux[1] its reciprocal (for the look-ahead bound of lookahead.h) */
static void chopper_aux(const RampComp& c, float* aux) {
  aux[0] = 2.0f * RC_PI / (float)(uint32_t)c.si[0];
  aux[1] = 1.0f / aux[0];
}

/* Convert one caller descriptor into its device form.  Tables (and a mesh's
 * BVH) are uploaded when the plan does not hold them yet; with may_upload
 * false they must already be held (callers that may not allocate). */
static int make_comp(RampPlan* p, const RampComp& c, CompDev& d, HashMemo* memo = nullptr,
                     bool may_upload = true) {
  memset(&d, 0, sizeof(d));
  d.geom = c.geom; d.scat = c.scat; d.idx = c.idx; d.restore = c.restore;
  memcpy(d.pos, c.pos, sizeof(d.pos));
  rot_matrix(c.rot, d.R);
  d.rotated = (c.rot[0] != 0.0f || c.rot[1] != 0.0f || c.rot[2] != 0.0f);
  memcpy(d.gp, c.gp, sizeof(d.gp));
  memcpy(d.sp, c.sp, sizeof(d.sp));
  memcpy(d.gi, c.gi, sizeof(d.gi));
  memcpy(d.si, c.si, sizeof(d.si));
  for (int k = 0; k < 6; ++k) d.dslot[k] = -1;
  d.priv_off = -1;
  if (c.scat == RAMP_S_GUIDE) guide_aux(c, d.aux);
  if (c.scat == RAMP_S_CHOPPER) chopper_aux(c, d.aux);   /* no slits: period inf, as 2 pi / 0 */
  for (int k = 0; k < RAMP_NTAB; ++k) {
    d.tab_len[k] = c.table_len[k];
    if (c.geom == RAMP_G_MESH && k == 0) continue;   /* the BVH replaces the raw points */
    int rc = may_upload ? get_table(p, c.table[k], c.table_len[k], &d.tab[k], memo)
                        : lookup_table(p, c.table[k], c.table_len[k], &d.tab[k], memo);
    if (rc) {
      if (!may_upload)
        set_err("table %d of a component is not held by the plan (create the plan from a "
                "variant with the same tables)", k);
      return rc;
    }
  }
  d.tally = c.tally;
  d.tally_err = c.tally_err;
  d.tally_len = c.tally_len;
  if (c.geom == RAMP_G_MESH) {
    int rc = may_upload ? get_bvh(p, c.table[0], c.table_len[0], &d.bvh_nodes, &d.bvh_tris, memo)
                        : lookup_bvh(p, c.table[0], c.table_len[0], &d.bvh_nodes, &d.bvh_tris,
                                     memo);
    if (rc) return rc;
  }
  return RAMP_OK;
}

static int check_state(const RampState* st, int64_t n) {
  if (!st || !st->soa || !st->iidx) { set_err("state pointers are NULL"); return RAMP_E_INVALID; }
  if (st->stride < n) { set_err("state stride %lld < n %lld", (long long)st->stride, (long long)n); return RAMP_E_INVALID; }
  return RAMP_OK;
}

static PlainArgs plain_args(RampPlan* p, const RampState* st, int64_t n, const RampRng* rng) {
  PlainArgs a;
  a.soa = st->soa;
  a.iidx = st->iidx;
  a.stride = st->stride;
  a.n = n;
  a.rng.mode = rng ? rng->mode : 0;
  a.rng.run_seed = rng ? rng->run_seed : 0u;
  a.rng.one = 1u;
  a.rng.tid_base = rng ? rng->tid_base : 0u;
  a.rng.seed_dev = rng ? rng->seed_dev : nullptr;
  a.st = p->status;
  return a;
}

extern "C" {

int ramp_version(void) { return RAMP_ABI_VERSION; }

int ramp_last_error(char* buf, int len) {
  if (!buf || len <= 0) return RAMP_E_INVALID;
  snprintf(buf, (size_t)len, "%s", g_err.c_str());
  return RAMP_OK;
}

int ramp_plan_destroy(RampPlan* p) {
  if (!p) return RAMP_OK;
  if (!p->allocs.empty()) {
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != p->device) cudaSetDevice(p->device);
    cudaDeviceSynchronize();      /* as cudaFree would: no kernel reads them any more */
    plan_release(p->device, p->allocs);
    if (prev != p->device) cudaSetDevice(prev);
  }
  if (p->batch.comps_dev) cudaFree(p->batch.comps_dev);
  if (p->batch.vars_dev) cudaFree(p->batch.vars_dev);
  if (p->surv && p->surv_owned) cudaFree(p->surv);
  if (p->adj_list) cudaFree(p->adj_list);
  if (p->batch.counters) cudaFree(p->batch.counters);
  if (p->streams.ready) {
    for (int k = 0; k < RAMP_BATCH_STREAMS; ++k) {
      cudaStreamDestroy(p->streams.st[k]);
      cudaEventDestroy(p->streams.join[k]);
    }
    cudaEventDestroy(p->streams.fork);
  }
  delete p;
  return RAMP_OK;
}

int ramp_plan_create(const RampSource* source, const RampComp* comps, int n_comps,
                     const RampBlock* blocks, int n_blocks, RampPlan** out) {
  if (!out || !source || (n_comps > 0 && !comps) || n_comps < 0 || n_blocks < 0 ||
      (n_blocks > 0 && !blocks)) {
    set_err("ramp_plan_create: invalid arguments");
    return RAMP_E_INVALID;
  }
  *out = nullptr;
  RampPlan* p = new RampPlan();
  cudaGetDevice(&p->device);
  p->src_in = *source;
  int rc = make_src(p, *source, p->src);
  if (rc) { ramp_plan_destroy(p); return rc; }   /* frees any table it uploaded */
  for (int b = 0; b < n_blocks; ++b) {
    const RampBlock& B = blocks[b];
    if (B.first < 0 || B.count < 0 || B.first + B.count > n_comps || (!B.linear && B.multi < 0)) {
      set_err("block %d covers components outside [0, %d)", b, n_comps);
      ramp_plan_destroy(p);
      return RAMP_E_INVALID;
    }
  }
  p->comps_in.assign(comps, comps + n_comps);
  p->blocks.assign(blocks, blocks + n_blocks);
  p->comps.resize((size_t)n_comps);
  for (int j = 0; j < n_comps; ++j) {
    rc = validate_comp(comps[j], j);
    if (!rc) rc = make_comp(p, comps[j], p->comps[j]);
    if (rc) { ramp_plan_destroy(p); return rc; }
  }
  for (const RampComp& c : p->comps_in) {
    if (c.scat == RAMP_S_RESCAL || c.scat == RAMP_S_HOST) p->plain_only = true;
    if (c.scat == RAMP_S_MONO || c.scat == RAMP_S_POWDER1) p->ext = true;
    if (c.geom == RAMP_G_MESH || c.scat == RAMP_S_ATTENUATE) p->mesh = true;
  }
  if (ext_source(*source)) p->ext = true;
  for (const RampBlock& B : p->blocks)
    for (int j = B.first; !B.linear && j < B.first + B.count; ++j)
      if (p->comps_in[j].scat == RAMP_S_RESCAL || p->comps_in[j].scat == RAMP_S_HOST) {
        set_err("component %d: SRescal and host components must sit in a linear block", j);
        ramp_plan_destroy(p);
        return RAMP_E_UNSUPPORTED;
      }
  void* d;
  rc = upload(p->comps.data(), p->comps.size() * sizeof(CompDev), &d, p->allocs);
  if (rc) { ramp_plan_destroy(p); return rc; }
  p->comps_dev = (CompDev*)d;
  rc = upload(p->blocks.data(), p->blocks.size() * sizeof(RampBlock), &d, p->allocs);
  if (rc) { ramp_plan_destroy(p); return rc; }
  p->blocks_dev = (RampBlock*)d;
  StatusDev zero;
  memset(&zero, 0, sizeof(zero));
  rc = upload(&zero, sizeof(zero), &d, p->allocs);
  if (rc) { ramp_plan_destroy(p); return rc; }
  p->status = (StatusDev*)d;
  cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, p->device);
  if (p->sm_count <= 0) p->sm_count = 1;
  *out = p;
  return RAMP_OK;
}

int ramp_plan_status(RampPlan* p, uint32_t* flags, uint64_t* oob) {
  if (!p) { set_err("NULL plan"); return RAMP_E_INVALID; }
  StatusDev h;
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(&h, p->status, sizeof(h), cudaMemcpyDeviceToHost));
  CK(cudaMemset(p->status, 0, sizeof(StatusDev)));
  if (flags) *flags = h.flags;
  if (oob) *oob = h.oob;
  return RAMP_OK;
}

int ramp_generate(RampPlan* p, const RampState* st, int64_t n, int32_t num_sim, int32_t seed,
                  const RampRng* rng, void* stream) {
  if (!p) { set_err("NULL plan"); return RAMP_E_INVALID; }
  int rc = check_state(st, n);
  if (rc) return rc;
  CK(launch_generate(p->src, plain_args(p, st, n, rng), num_sim, seed, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_run_block(RampPlan* p, int block, const RampState* st, int64_t n, const RampRng* rng,
                   void* stream) {
  if (!p || block < 0 || block >= (int)p->blocks.size()) {
    set_err("ramp_run_block: bad plan or block index");
    return RAMP_E_INVALID;
  }
  int rc = check_state(st, n);
  if (rc) return rc;
  const RampBlock& B = p->blocks[block];
  PlainArgs a = plain_args(p, st, n, rng);
  cudaStream_t s = (cudaStream_t)stream;
  if (B.linear) {
    for (int j = B.first; j < B.first + B.count; ++j) CK(launch_linear_comp(p->comps[j], a, s));
  } else {
    bool mesh = false;
    for (int j = B.first; j < B.first + B.count; ++j) mesh = mesh || p->comps[j].geom == RAMP_G_MESH;
    CK(launch_nonlinear_block(p->comps_dev, B.first, B.count, B.multi, mesh, a, s));
  }
  return RAMP_OK;
}

int ramp_trace_plain(RampPlan* p, const RampState* st, int64_t n, int32_t num_sim, int32_t seed,
                     const RampRng* rng, void* stream) {
  int rc = ramp_generate(p, st, n, num_sim, seed, rng, stream);
  if (rc) return rc;
  for (int b = 0; b < (int)p->blocks.size(); ++b) {
    rc = ramp_run_block(p, b, st, n, rng, stream);
    if (rc) return rc;
  }
  return RAMP_OK;
}

/* persistent grid for the fused kernel: one CTA per span at most */
static int fused_grid(int64_t n_spans, int grid) {
  int64_t need = n_spans < 1 ? 1 : n_spans;
  return (int)(need < grid ? need : grid);
}

/* CTAs per row of a batched launch: enough for the longest variant to give
 * every warp one work item (rows of shorter variants leave the rest idle
 * at once), at most one resident grid */
static int batched_grid(int64_t n_max, int grid) {
  return fused_grid((n_max + 8 * 128 - 1) / (8 * 128), grid);
}

static void tune_defaults(RampPlan* p, const RampTune* tune, int& block, int& grid,
                          int64_t& task, int32_t& minb) {
  /* CTAs of 256 threads, or 128 on request (the kernels are compiled for
     at most 256 threads a CTA) */
  block = (tune && tune->block == 128) ? 128 : 256;
  /* register cap (minimum 256-thread CTAs per SM the kernel is compiled
     for): 4 by default, the fastest measured on GB300 for every chain
     tried (single, split, batched); 3 when fewer than 4 x 256 threads per
     SM are asked for */
  minb = (tune && tune->blocks_per_sm > 0 && tune->blocks_per_sm * block < 4 * 256) ? 3 : 4;
  int bps = (tune && tune->blocks_per_sm > 0) ? tune->blocks_per_sm
                                              : fused_max_blocks_per_sm(block, minb);
  grid = p->sm_count * bps;
  task = (tune && tune->chunk > 0) ? tune->chunk : 0;   /* 0: auto_task() */
}

/* survivor-compaction point of a fused launch (RampTune.split): a
 * component index in [0, n_comps) not strictly inside a non-linear block */
static int tune_split(const RampPlan* p, const RampTune* tune, int32_t* out) {
  *out = 0;
  if (!tune || tune->split <= 0) return RAMP_OK;
  const int k = tune->split;
  if (k >= (int)p->comps.size()) {
    set_err("RampTune.split %d: the chain has %d components", k, (int)p->comps.size());
    return RAMP_E_INVALID;
  }
  for (const RampBlock& B : p->blocks)
    if (!B.linear && B.first < k && k < B.first + B.count) {
      set_err("RampTune.split %d falls inside a non-linear block", k);
      return RAMP_E_INVALID;
    }
  *out = k;
  return RAMP_OK;
}

/* ---- chopper look-ahead (RampTune.cull; the bound is in lookahead.h) ---- */
static bool on_axis_plane(const RampComp& c) {
  return c.geom == RAMP_G_PLANE && c.gi[0] == 0 && c.restore == 0 && c.rot[0] == 0.0f &&
         c.rot[1] == 0.0f && c.rot[2] == 0.0f && c.pos[0] == 0.0f && c.pos[1] == 0.0f &&
         std::isfinite(c.pos[2]);
}

/* length of the run of on-axis components at k: straight guides and disk
 * choppers in any order, non-overlapping at non-decreasing z, up to the
 * last chopper before the first component that is neither (0: no
 * chopper); when the component right after that chopper is an on-axis,
 * unrotated GCylinderExt without restore that starts beyond it, the run
 * takes it as its target (its last component) */
static int chopper_run(const RampComp* comps, int nc, const RampBlock* blocks, int nb, int k) {
  if (!comps || !blocks || k < 0 || k >= nc) return 0;
  int end = -1;
  for (int b = 0; b < nb; ++b)
    if (blocks[b].linear && blocks[b].first <= k && k < blocks[b].first + blocks[b].count)
      end = std::min(blocks[b].first + blocks[b].count, nc);
  if (end < 0) return 0;
  float zmin = -INFINITY;
  int last = -1;
  for (int j = k; j < end; ++j) {
    const RampComp& c = comps[j];
    if (!on_axis_plane(c) || !(c.pos[2] >= zmin)) break;
    if (c.scat == RAMP_S_GUIDE) {
      if (!(c.sp[0] == c.sp[2]) || !(c.sp[1] == c.sp[3]) || !(c.sp[0] > 0.0f) ||
          !(c.sp[1] > 0.0f) || !(c.sp[4] > 0.0f) || !std::isfinite(c.sp[4]) ||
          !std::isfinite(c.sp[0]) || !std::isfinite(c.sp[1]) || !(c.gp[0] > 0.0f) ||
          !(c.gp[1] > 0.0f))
        break;
      zmin = c.pos[2] + c.sp[4];
    } else if (c.scat == RAMP_S_CHOPPER) {
      bool finite = true;
      for (int q = 0; q < 5; ++q) finite = finite && std::isfinite(c.sp[q]);
      if (!finite || !(c.sp[1] > 0.0f) || (uint32_t)c.si[0] == 0u) break;
      zmin = c.pos[2];
      last = j;
    } else {
      break;
    }
  }
  if (last < 0) return 0;
  if (last + 1 < end) {
    const RampComp& c = comps[last + 1];
    if (c.geom == RAMP_G_CYL_EXT && c.restore == 0 && c.rot[0] == 0.0f && c.rot[1] == 0.0f &&
        c.rot[2] == 0.0f && c.pos[0] == 0.0f && c.pos[1] == 0.0f && std::isfinite(c.pos[2]) &&
        c.gp[0] > 0.0f && std::isfinite(c.gp[0]) && c.gp[1] > 0.0f && std::isfinite(c.gp[1]) &&
        c.pos[2] - c.gp[0] >= comps[last].pos[2])
      return last - k + 2;
  }
  return last - k + 1;
}

/* the launch's stage split: RampTune.cull (split before component
 * `split`, which may be 0, and retire in stage A what the look-ahead
 * shows cannot pass the chopper run there; every variant must hold the
 * run), else RampTune.walk (chains without the extended kinds that hold a
 * GMesh component in a linear block: split before the first such
 * component, which may be component 0, and walk the mesh per lane in
 * stage B), else RampTune.split */
static int tune_stage(const RampPlan* p, const RampTune* tune, bool ext, int32_t* split,
                      int32_t* walk, int32_t* cull, const RampVariant* vars = nullptr,
                      int n_vars = 0) {
  *walk = 0;
  *cull = 0;
  if (tune && tune->cull > 0) {
    if (tune->walk > 0) {
      set_err("RampTune.cull and RampTune.walk exclude each other");
      return RAMP_E_INVALID;
    }
    const int nc = (int)p->comps.size();
    const int k = tune->split > 0 ? tune->split : 0;
    int nl = chopper_run(p->comps_in.data(), nc, p->blocks.data(), (int)p->blocks.size(), k);
    for (int v = 0; v < n_vars && nl > 0; ++v)
      nl = std::min(nl, chopper_run(vars[v].comps, nc, p->blocks.data(), (int)p->blocks.size(), k));
    if (nl == 0) {
      set_err("RampTune.cull: no run of on-axis straight guides and choppers "
              "starts at component %d", k);
      return RAMP_E_INVALID;
    }
    *split = k;
    *cull = nl;
    return RAMP_OK;
  }
  if (tune && tune->walk > 0 && !ext) {
    for (const RampBlock& B : p->blocks) {
      if (!B.linear) continue;
      for (int k = B.first; k < B.first + B.count; ++k)
        if (p->comps[k].geom == RAMP_G_MESH) {
          *split = k;
          *walk = 1;
          return RAMP_OK;
        }
    }
  }
  return tune_split(p, tune, split);
}

/* The descriptors of a whole-chain launch with private tallies
 * (RampTune.privatize): detectors (SDetector1D, SDetector2D) whose two
 * histograms fit in what is left of RAMP_PRIV_FLOATS shared-memory floats
 * get an offset there, in chain order; the copy goes to a plan-owned
 * device array.  Returns the floats used (0: none fits, nothing to do). */
static int priv_descriptors(RampPlan* p, cudaStream_t s, int32_t* floats) {
  *floats = 0;
  std::vector<CompDev> c = p->comps;
  int used = 0;
  for (CompDev& d : c) {
    if (d.scat != RAMP_S_DET1D && d.scat != RAMP_S_DET2D) continue;
    if (!d.tally || !d.tally_err || d.tally_len <= 0) continue;
    const int64_t need = 2 * d.tally_len;
    if (used + need > RAMP_PRIV_FLOATS) continue;
    d.priv_off = used;
    used += (int)need;
  }
  if (used == 0) return RAMP_OK;
  if (!p->priv_dev) {
    void* d = nullptr;
    cudaError_t e = plan_alloc(c.size() * sizeof(CompDev), &d, p->allocs);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_err("private-tally descriptors: %s", cudaGetErrorString(e));
      return RAMP_E_NOMEM;
    }
    p->priv_dev = (CompDev*)d;
  }
  /* pageable source: the copy is staged before cudaMemcpyAsync returns */
  cudaError_t e = cudaMemcpyAsync(p->priv_dev, c.data(), c.size() * sizeof(CompDev),
                                  cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    set_err("private-tally descriptors: %s", cudaGetErrorString(e));
    return RAMP_E_CUDA;
  }
  *floats = used;
  return RAMP_OK;
}

/* bytes of the survivor buffer for n_items work items of 128 neutrons:
 * SURV_WORDS_WALK words per slot (the record and, after a mesh walk, its
 * result) plus one count per item */
static size_t surv_bytes(int64_t n_items) {
  return ((size_t)n_items * 128 * SURV_WORDS_WALK + (size_t)n_items) * sizeof(uint32_t);
}

/* survivor buffer for split launches covering up to n_items work items:
 * the caller's (ramp_plan_set_survivors) when it is large enough, else one
 * of the plan's own (grows, never shrinks) */
static int ensure_surv(RampPlan* p, int64_t n_items) {
  const int64_t slots = n_items * 128;
  if (p->surv_ext && surv_bytes(n_items) <= (size_t)p->surv_ext_bytes) {
    if (p->surv && p->surv_owned) cudaFree(p->surv);
    p->surv = p->surv_ext;
    p->surv_cap = slots;
    p->surv_owned = false;
    return RAMP_OK;
  }
  if (p->surv && p->surv_owned && slots <= p->surv_cap) return RAMP_OK;
  if (p->surv && p->surv_owned) cudaFree(p->surv);
  p->surv = nullptr;
  p->surv_cap = 0;
  p->surv_owned = false;
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, surv_bytes(n_items));
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_err("survivor buffer for %lld histories: %s", (long long)slots, cudaGetErrorString(e));
    return RAMP_E_NOMEM;
  }
  p->surv = (uint32_t*)d;
  p->surv_cap = slots;
  p->surv_owned = true;
  return RAMP_OK;
}

/* wire a split launch of n_items work items to the survivor buffer */
static int attach_surv(RampPlan* p, FusedArgs& a, int64_t n_items, cudaStream_t s) {
  int rc = ensure_surv(p, n_items);
  if (rc) return rc;
  a.surv = p->surv;
  a.surv_cap = p->surv_cap;
  a.surv_cnt = p->surv + (size_t)p->surv_cap * SURV_WORDS_WALK;
  a.surv_items = n_items;
  CK(cudaMemsetAsync(a.surv_cnt, 0, (size_t)n_items * sizeof(uint32_t), s));
  return RAMP_OK;
}

/* the linear block holding component k, or -1 */
static int linear_block_of(const RampPlan* p, int k) {
  for (size_t b = 0; b < p->blocks.size(); ++b) {
    const RampBlock& B = p->blocks[b];
    if (k >= B.first && k < B.first + B.count) return B.linear ? (int)b : -1;
  }
  return -1;
}

int ramp_run_components(RampPlan* p, int32_t k0, int32_t k1, const RampState* st, int64_t n,
                        const RampRng* rng, void* stream) {
  if (!p || k0 < 0 || k1 > (int)p->comps.size() || k0 > k1) {
    set_err("ramp_run_components: bad range");
    return RAMP_E_INVALID;
  }
  int rc = check_state(st, n);
  if (rc) return rc;
  PlainArgs a = plain_args(p, st, n, rng);
  for (int k = k0; k < k1; ++k) {
    if (linear_block_of(p, k) < 0) {
      set_err("ramp_run_components: component %d is not in a linear block", k);
      return RAMP_E_INVALID;
    }
    CK(launch_linear_comp(p->comps[k], a, (cudaStream_t)stream));
  }
  return RAMP_OK;
}

static int host_half(RampPlan* p, int32_t comp, const RampState* st, int64_t n,
                     const RampRng* rng, int leave, void* stream) {
  if (!p || comp < 0 || comp >= (int)p->comps.size() || linear_block_of(p, comp) < 0) {
    set_err("ramp_component_%s: component %d is not in a linear block", leave ? "leave" : "enter",
            comp);
    return RAMP_E_INVALID;
  }
  int rc = check_state(st, n);
  if (rc) return rc;
  CK(launch_host_half(p->comps[comp], plain_args(p, st, n, rng), leave, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_component_enter(RampPlan* p, int32_t comp, const RampState* st, int64_t n,
                         const RampRng* rng, void* stream) {
  return host_half(p, comp, st, n, rng, 0, stream);
}

int ramp_component_leave(RampPlan* p, int32_t comp, const RampState* st, int64_t n,
                         void* stream) {
  return host_half(p, comp, st, n, nullptr, 1, stream);
}

int ramp_gather_alive(const RampState* st, int64_t n, uint32_t lanes, float* out,
                      int64_t* scratch, int64_t scratch_len, int64_t* count, void* stream) {
  int rc = check_state(st, n);
  if (rc) return rc;
  if (!out || !count || lanes == 0 || lanes >= (1u << RAMP_NLANES) ||
      (n > 0 && (!scratch || scratch_len < (n + 1023) / 1024))) {
    set_err("ramp_gather_alive: bad arguments (scratch needs ceil(n/1024) entries)");
    return RAMP_E_INVALID;
  }
  PlainArgs a;
  memset(&a, 0, sizeof(a));
  a.soa = st->soa;
  a.iidx = st->iidx;
  a.stride = st->stride;
  a.n = n;
  CK(launch_gather_alive(a, lanes, out, scratch, count, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_plan_set_buffer(RampPlan* p, int32_t comp, float* buf, int64_t len) {
  if (!p || comp < 0 || comp >= (int)p->comps.size() || len < 0 || (len > 0 && !buf)) {
    set_err("ramp_plan_set_buffer: bad arguments");
    return RAMP_E_INVALID;
  }
  p->comps[comp].tally = buf;
  p->comps[comp].tally_len = len;
  p->comps_in[comp].tally = buf;
  p->comps_in[comp].tally_len = len;
  CK(cudaMemcpy(p->comps_dev + comp, &p->comps[comp], sizeof(CompDev), cudaMemcpyHostToDevice));
  return RAMP_OK;
}

int ramp_plan_reserve(RampPlan* p, int64_t n) {
  if (!p || n < 0) { set_err("ramp_plan_reserve: bad arguments"); return RAMP_E_INVALID; }
  return ensure_surv(p, (n + 127) / 128);
}

int64_t ramp_survivor_bytes(int64_t n) {
  return n > 0 ? (int64_t)surv_bytes((n + 127) / 128) : 0;
}

int ramp_plan_set_survivors(RampPlan* p, void* buf, int64_t bytes) {
  if (!p || bytes < 0 || (buf && ((uintptr_t)buf & 15))) {
    set_err("ramp_plan_set_survivors: a 16-byte aligned device buffer and its size");
    return RAMP_E_INVALID;
  }
  if (p->surv && !p->surv_owned) { p->surv = nullptr; p->surv_cap = 0; }
  p->surv_ext = buf ? (uint32_t*)buf : nullptr;
  p->surv_ext_bytes = buf ? bytes : 0;
  return RAMP_OK;
}

/* span size for n histories: about eight spans per resident CTA, in
 * multiples of 1024 neutrons, between 1024 and 65536 */
static int64_t auto_task(int64_t n, int grid, int64_t task) {
  if (task > 0) return task;
  int64_t t = n / ((int64_t)grid * 8);
  t = (t + 1023) / 1024 * 1024;
  if (t < 1024) t = 1024;
  if (t > 65536) t = 65536;
  return t;
}

int ramp_trace_fused(RampPlan* p, int64_t n, int32_t num_sim, int32_t seed, const RampRng* rng,
                     float* sb_carry, uint32_t* iidx_carry, const RampTune* tune, void* stream) {
  if ((sb_carry == nullptr) != (iidx_carry == nullptr)) {
    set_err("ramp_trace_fused: give both carry buffers or neither");
    return RAMP_E_INVALID;
  }
  if (!p || n < 0) { set_err("ramp_trace_fused: bad arguments"); return RAMP_E_INVALID; }
  if (int rc0 = check_whole_chain(p, "ramp_trace_fused")) return rc0;
  if ((int)p->comps.size() > RAMP_MAX_COMPS) {
    set_err("fused path supports at most %d components", RAMP_MAX_COMPS);
    return RAMP_E_RANGE;
  }
  if (n == 0) return RAMP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int block, grid;
  int64_t task;
  int32_t minb;
  tune_defaults(p, tune, block, grid, task, minb);
  task = auto_task(n, grid, task);
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.minb = minb;
  a.variants = nullptr;
  a.task_size = task;
  a.n_tasks = (n + task - 1) / task;
  a.single.src = p->src;
  a.single.n = n;
  a.single.num_sim = num_sim;
  a.single.seed = seed;
  a.single.comps = p->comps_dev;
  a.blocks = p->blocks_dev;
  a.n_blocks = (int32_t)p->blocks.size();
  a.n_comps = (int32_t)p->comps.size();
  a.rng.mode = rng ? rng->mode : 0;
  a.rng.run_seed = rng ? rng->run_seed : 0u;
  a.rng.one = 1u;
  a.rng.tid_base = rng ? rng->tid_base : 0u;
  a.rng.seed_dev = rng ? rng->seed_dev : nullptr;
  a.carry_sb = sb_carry;
  a.carry_iidx = iidx_carry;
  a.st = p->status;
  a.workq = &p->status->workq;
  a.workq_b = &p->status->workq_b;
  a.workq_c = &p->status->workq_c;
  int rc = tune_stage(p, tune, p->ext, &a.split, &a.walk, &a.cull);
  if (!rc && tune && tune->privatize > 0 && a.split == 0 && !a.walk && !a.cull) {
    rc = priv_descriptors(p, s, &a.priv_floats);
    if (!rc && a.priv_floats > 0) a.single.comps = p->priv_dev;
  }
  if (rc) return rc;
  a.ext = kind_set(p->ext, p->mesh);
  if (a.split > 0 || a.walk || a.cull) {
    rc = attach_surv(p, a, (n + 127) / 128, s);
    if (rc) return rc;
  }
  /* workq, surv, workq_b and workq_c */
  CK(cudaMemsetAsync(&p->status->workq, 0, 4 * sizeof(unsigned long long), s));
  CK(launch_fused(a, block, fused_grid(a.n_tasks, grid), s));
  return RAMP_OK;
}

/* ramp_trace_batched as concurrent single-variant launches: each variant
 * is a launch of the single-instrument kernel (its descriptors are kernel
 * parameters, read through the uniform datapath) with its own work-queue
 * counter, spread longest-first over RAMP_BATCH_STREAMS streams that fork
 * from and join back into the caller's stream (event record/wait only, so
 * the whole call can be captured in a CUDA graph).  Kernels of different
 * streams fill each other's tails. */
static int batched_streams(RampPlan* p, FusedArgs base, const std::vector<VariantDev>& vars,
                           int block, int grid, const RampTune* tune, int32_t split,
                           int32_t walk, int32_t cull, cudaStream_t s) {
  BatchCache& B = p->batch;
  const size_t nv = vars.size();
  if (B.counters_cap < 3 * nv) {   /* stage A, stage B and walk-finishing queues */
    if (B.counters) cudaFree(B.counters);
    B.counters = nullptr;
    B.counters_cap = 0;
    CK(cudaMalloc(&B.counters, 3 * nv * sizeof(unsigned long long)));
    B.counters_cap = 3 * nv;
  }
  /* split launches: each variant gets its own region of the survivor
     buffer (its items' slots, SoA, and its items' counts) */
  int rc0 = RAMP_OK;
  std::vector<int64_t> item_off(nv + 1, 0);
  for (size_t v = 0; v < nv; ++v)
    item_off[v + 1] = item_off[v] + (vars[v].n > 0 ? (vars[v].n + 127) / 128 : 0);
  uint32_t* cnt = nullptr;
  if ((split > 0 || walk || cull) && item_off[nv] > 0) {
    rc0 = ensure_surv(p, item_off[nv]);
    if (rc0) return rc0;
    cnt = p->surv + (size_t)p->surv_cap * SURV_WORDS_WALK;
    CK(cudaMemsetAsync(cnt, 0, (size_t)item_off[nv] * sizeof(uint32_t), s));
  }
  StreamSet& S = p->streams;
  if (!S.ready) {
    for (int k = 0; k < RAMP_BATCH_STREAMS; ++k) {
      CK(cudaStreamCreateWithFlags(&S.st[k], cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&S.join[k], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming));
    S.ready = true;
  }
  const int ns = (tune && tune->streams > 1 && tune->streams < RAMP_BATCH_STREAMS)
                     ? tune->streams : RAMP_BATCH_STREAMS;
  CK(cudaMemsetAsync(B.counters, 0, 3 * nv * sizeof(unsigned long long), s));
  CK(cudaEventRecord(S.fork, s));
  for (int k = 0; k < ns; ++k) CK(cudaStreamWaitEvent(S.st[k], S.fork, 0));
  std::vector<int> order(nv);
  for (size_t v = 0; v < nv; ++v) order[v] = (int)v;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return vars[x].n > vars[y].n; });
  std::vector<int64_t> load(ns, 0);
  for (int v : order) {
    if (vars[v].n <= 0) continue;
    int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += vars[v].n;
    FusedArgs a = base;
    a.variants = nullptr;
    a.single = vars[v];
    a.var_key = v;
    a.workq = B.counters + v;
    a.workq_b = B.counters + nv + v;
    a.workq_c = B.counters + 2 * nv + v;
    a.task_size = auto_task(vars[v].n, grid, 0);
    a.n_tasks = (vars[v].n + a.task_size - 1) / a.task_size;
    if (cnt) {
      const int64_t items = item_off[v + 1] - item_off[v];
      a.split = split;
      a.walk = walk;
      a.cull = cull;
      a.surv = p->surv + (size_t)item_off[v] * 128 * SURV_WORDS_WALK;
      a.surv_cap = items * 128;
      a.surv_cnt = cnt + item_off[v];
      a.surv_items = items;
    }
    CK(launch_fused(a, block, fused_grid(a.n_tasks, grid), S.st[k]));
  }
  for (int k = 0; k < ns; ++k) {
    CK(cudaEventRecord(S.join[k], S.st[k]));
    CK(cudaStreamWaitEvent(s, S.join[k], 0));
  }
  return RAMP_OK;
}

int ramp_trace_batched(RampPlan* p, const RampVariant* variants, int n_variants,
                       const RampRng* rng, const RampTune* tune, void* stream) {
  if (!p || !variants || n_variants <= 0) {
    set_err("ramp_trace_batched: bad arguments");
    return RAMP_E_INVALID;
  }
  if (int rc0 = check_whole_chain(p, "ramp_trace_batched")) return rc0;
  const int nc = (int)p->comps.size();
  if (nc > RAMP_MAX_COMPS) {
    set_err("fused path supports at most %d components", RAMP_MAX_COMPS);
    return RAMP_E_RANGE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int block, grid;
  int64_t task;
  int32_t minb;
  tune_defaults(p, tune, block, grid, task, minb);
  {
    int64_t total = 0;
    for (int v = 0; v < n_variants; ++v) total += variants[v].n > 0 ? variants[v].n : 0;
    task = auto_task(total, grid, task);
  }
  BatchCache& B = p->batch;
  /* descriptors: re-upload only when they change */
  std::vector<CompDev> comps((size_t)n_variants * nc);
  HashMemo memo;
  for (int v = 0; v < n_variants; ++v) {
    if (!variants[v].comps || variants[v].n < 0) {
      set_err("variant %d: missing components", v);
      return RAMP_E_INVALID;
    }
    for (int j = 0; j < nc; ++j) {
      const RampComp& c = variants[v].comps[j];
      if (c.geom != p->comps_in[j].geom || c.scat != p->comps_in[j].scat) {
        set_err("variant %d component %d: kinds differ from the plan", v, j);
        return RAMP_E_INVALID;
      }
      int rc = validate_comp(c, j);
      if (!rc) rc = make_comp(p, c, comps[(size_t)v * nc + j], &memo);
      if (rc) return rc;
    }
  }
  size_t cbytes = comps.size() * sizeof(CompDev);
  if (B.comps_cap < comps.size()) {
    if (B.comps_dev) cudaFree(B.comps_dev);
    CK(cudaMalloc(&B.comps_dev, cbytes));
    B.comps_cap = comps.size();
    B.comps_host.clear();
  }
  if (B.comps_host.size() != comps.size() ||
      memcmp(B.comps_host.data(), comps.data(), cbytes) != 0) {
    CK(cudaMemcpy(B.comps_dev, comps.data(), cbytes, cudaMemcpyHostToDevice));
    B.comps_host = comps;
  }
  std::vector<VariantDev> vars((size_t)n_variants);
  /* default: one launch with a grid row per variant; streams >= 2: one
     launch per variant over that many concurrent streams */
  const bool use_streams = tune && tune->streams > 1;
  int64_t n_max = 0;
  for (int v = 0; v < n_variants; ++v) {
    int rc = make_src(p, variants[v].source, vars[v].src, true, &memo);
    if (rc) return rc;
    vars[v].n = variants[v].n;
    vars[v].num_sim = variants[v].num_sim;
    vars[v].seed = variants[v].seed;
    vars[v].comps = B.comps_dev + (size_t)v * nc;
    if (vars[v].n > n_max) n_max = vars[v].n;
  }
  bool ext = p->ext;
  for (int v = 0; v < n_variants; ++v) ext = ext || ext_source(variants[v].source);
  int32_t split = 0, walk = 0, cull = 0;
  if (int rc = tune_stage(p, tune, ext, &split, &walk, &cull, variants, n_variants)) return rc;
  if (use_streams) {
    FusedArgs a;
    memset(&a, 0, sizeof(a));
    a.minb = minb;
    a.ext = kind_set(ext, p->mesh);
    a.blocks = p->blocks_dev;
    a.n_blocks = (int32_t)p->blocks.size();
    a.n_comps = nc;
    a.rng.mode = rng ? rng->mode : 1;
    a.rng.run_seed = rng ? rng->run_seed : 0u;
    a.rng.one = 1u;
    a.rng.tid_base = 0u;   /* variants key by their own index */
    a.st = p->status;
    return batched_streams(p, a, vars, block, grid, tune, split, walk, cull, s);
  }
  /* one launch: grid row v traces variant v from its own work counter
     (two with a split), its survivors in its own range of work items */
  if (n_variants > 65535) {
    set_err("ramp_trace_batched: %d variants in one launch (at most 65535; use streams)",
            n_variants);
    return RAMP_E_RANGE;
  }
  if (n_max == 0) return RAMP_OK;
  int rc = RAMP_OK;
  if (ext) split = cull = 0;   /* the one-launch kernel runs the extended kinds whole */
  int64_t items = 0;
  for (int v = 0; v < n_variants; ++v) {
    vars[v].item_off = items;
    items += (vars[v].n + 127) / 128;
  }
  if (B.vars_cap < vars.size()) {
    if (B.vars_dev) cudaFree(B.vars_dev);
    B.vars_dev = nullptr;
    B.vars_cap = 0;
    CK(cudaMalloc(&B.vars_dev, vars.size() * sizeof(VariantDev)));
    B.vars_cap = vars.size();
    B.vars_host.clear();
  }
  if (B.vars_host.size() != vars.size() ||
      memcmp(B.vars_host.data(), vars.data(), vars.size() * sizeof(VariantDev)) != 0) {
    CK(cudaMemcpy(B.vars_dev, vars.data(), vars.size() * sizeof(VariantDev),
                  cudaMemcpyHostToDevice));
    B.vars_host = vars;
  }
  if (B.counters_cap < 3 * (size_t)n_variants) {
    if (B.counters) cudaFree(B.counters);
    B.counters = nullptr;
    B.counters_cap = 0;
    CK(cudaMalloc(&B.counters, 3 * (size_t)n_variants * sizeof(unsigned long long)));
    B.counters_cap = 3 * (size_t)n_variants;
  }
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.minb = minb;
  a.variants = B.vars_dev;
  a.n_variants = n_variants;
  a.blocks = p->blocks_dev;
  a.n_blocks = (int32_t)p->blocks.size();
  a.n_comps = nc;
  a.rng.mode = rng ? rng->mode : 1;
  a.rng.run_seed = rng ? rng->run_seed : 0u;
  a.rng.one = 1u;
  a.rng.tid_base = 0u;   /* variants key by their own index */
  a.st = p->status;
  a.workq = B.counters;
  a.workq_b = B.counters + n_variants;
  a.workq_c = B.counters + 2 * n_variants;
  a.split = split;
  a.walk = walk;
  a.cull = cull;
  a.ext = kind_set(ext, p->mesh);
  if (a.split > 0 || a.walk || a.cull) {
    rc = attach_surv(p, a, items, s);
    if (rc) return rc;
  }
  CK(cudaMemsetAsync(B.counters, 0, 3 * (size_t)n_variants * sizeof(unsigned long long), s));
  CK(launch_fused(a, block, batched_grid(n_max, grid), s));
  return RAMP_OK;
}

int ramp_plan_set_param(RampPlan* p, int32_t kind, int32_t comp, float value) {
  if (!p) { set_err("NULL plan"); return RAMP_E_INVALID; }
  if (kind == RAMP_DP_SOURCE_T) {
    if (p->src_in.kind != RAMP_SRC_CONT) {
      set_err("ramp_plan_set_param: the source has no temperature");
      return RAMP_E_INVALID;
    }
    if (p->src_in.p[7] == value && p->src_in.p[9] == value && p->src_in.p[11] == value)
      return RAMP_OK;                      /* unchanged: nothing to do */
    p->src_in.p[7] = p->src_in.p[9] = p->src_in.p[11] = value;
    p->param_version++;
    return make_src(p, p->src_in, p->src);
  }
  if (comp < 0 || comp >= (int)p->comps_in.size()) {
    set_err("ramp_plan_set_param: component %d out of range", comp);
    return RAMP_E_INVALID;
  }
  RampComp& c = p->comps_in[comp];
  float* slot = nullptr;
  if (kind >= RAMP_DP_GUIDE_R0 && kind <= RAMP_DP_GUIDE_W) {
    if (c.scat != RAMP_S_GUIDE) { set_err("component %d is not a guide", comp); return RAMP_E_INVALID; }
    slot = &c.sp[5 + (kind - RAMP_DP_GUIDE_R0)];
  } else if (kind == RAMP_DP_POWDER_SIGMA_ABS) {
    if (c.scat != RAMP_S_POWDERN) { set_err("component %d is not a powder", comp); return RAMP_E_INVALID; }
    slot = &c.sp[0];
  } else {
    set_err("ramp_plan_set_param: unknown parameter kind %d", kind);
    return RAMP_E_INVALID;
  }
  if (memcmp(slot, &value, sizeof(float)) == 0) return RAMP_OK;   /* unchanged */
  *slot = value;
  p->param_version++;
  int rc = make_comp(p, c, p->comps[comp]);
  if (rc) return rc;
  CK(cudaMemcpy(p->comps_dev + comp, &p->comps[comp], sizeof(CompDev), cudaMemcpyHostToDevice));
  return RAMP_OK;
}

/* the adjoint's descriptor copy: derivative slots of params (may be none),
 * the loss detector marked */
static int prep_adjoint(RampPlan* p, const RampDiffParam* params, int n_params, int det_comp,
                        const float* dL_dH, SrcDev& src, cudaStream_t s) {
  const int nc = (int)p->comps.size();
  if (det_comp < 0 || det_comp >= nc ||
      (p->comps[det_comp].scat != RAMP_S_DET2D && p->comps[det_comp].scat != RAMP_S_DET1D)) {
    set_err("ramp_adjoint: component %d is not a histogram detector", det_comp);
    return RAMP_E_INVALID;
  }
  if ((int)p->adj_host.size() != nc) {
    p->adj_host.resize((size_t)nc);
    void* d;
    int rc = upload(p->comps.data(), (size_t)nc * sizeof(CompDev), &d, p->allocs);
    if (rc) return rc;
    p->adj_dev = (CompDev*)d;
  }
  std::vector<CompDev>& A = p->adj_host;
  A = p->comps;
  src = p->src;
  for (int k = 0; k < n_params; ++k) {
    const RampDiffParam& q = params[k];
    if (q.kind == RAMP_DP_SOURCE_T) {
      if (src.kind != RAMP_SRC_CONT) { set_err("ramp_adjoint: source has no temperature"); return RAMP_E_INVALID; }
      src.dslot_T = k;
      continue;
    }
    if (q.comp < 0 || q.comp >= nc) { set_err("ramp_adjoint: parameter %d: bad component", k); return RAMP_E_INVALID; }
    CompDev& c = A[q.comp];
    if (q.kind >= RAMP_DP_GUIDE_R0 && q.kind <= RAMP_DP_GUIDE_W && c.scat == RAMP_S_GUIDE) {
      c.dslot[q.kind - RAMP_DP_GUIDE_R0] = (int16_t)k;
    } else if (q.kind == RAMP_DP_POWDER_SIGMA_ABS && c.scat == RAMP_S_POWDERN) {
      c.dslot[0] = (int16_t)k;
    } else {
      set_err("ramp_adjoint: parameter %d (kind %d) does not match component %d", k, q.kind, q.comp);
      return RAMP_E_INVALID;
    }
  }
  A[det_comp].adj_det = 1;
  A[det_comp].dLdH = dL_dH;
  CK(cudaMemcpyAsync(p->adj_dev, A.data(), (size_t)nc * sizeof(CompDev), cudaMemcpyHostToDevice, s));
  return RAMP_OK;
}

/* arguments of an adjoint launch over n neutrons, with the index list */
static int adjoint_args(RampPlan* p, const SrcDev& src, int n_params, int64_t n, int32_t num_sim,
                        int32_t seed, const RampRng* rng, int lr, double* grad, AdjointArgs& a,
                        int& grid) {
  memset(&a, 0, sizeof(a));
  a.src = src;
  a.comps = p->adj_dev;
  a.blocks = p->blocks_dev;
  a.n_blocks = (int32_t)p->blocks.size();
  a.nslot = n_params;
  a.n = n;
  a.num_sim = num_sim;
  a.seed = seed;
  a.rng.mode = rng ? rng->mode : 0;
  a.rng.run_seed = rng ? rng->run_seed : 0u;
  a.rng.one = 1u;
  a.rng.tid_base = rng ? rng->tid_base : 0u;
  a.rng.seed_dev = rng ? rng->seed_dev : nullptr;
  a.grad = grad;
  a.lr = lr;
  a.st = p->status;
  a.cull = chopper_run(p->comps_in.data(), (int)p->comps.size(), p->blocks.data(),
                       (int)p->blocks.size(), 0);
  if (p->adj_cap < n) {   /* two lists of n indices (counted, kept), three
                             counters and the keep pass's speed table */
    if (p->adj_list) cudaFree(p->adj_list);
    p->adj_list = nullptr;
    p->adj_cap = 0;
    void* d = nullptr;
    if (cudaMalloc(&d, 2 * (size_t)n * sizeof(uint32_t) + 3 * sizeof(unsigned long long) +
                           sizeof(SpeedTab)) != cudaSuccess) {
      cudaGetLastError();
      set_err("ramp_adjoint: no room for %lld recorded indices", (long long)n);
      return RAMP_E_NOMEM;
    }
    p->adj_list = (uint32_t*)d;
    p->adj_cap = n;
    p->rec_valid = false;
  }
  a.list = p->adj_list;
  a.list_cap = p->adj_cap;
  a.keep = p->adj_list + p->adj_cap;
  a.list_count = (unsigned long long*)(((uintptr_t)(p->adj_list + 2 * p->adj_cap) + 7) &
                                       ~(uintptr_t)7);
  a.keep_count = a.list_count + 1;
  int64_t g = (n + 255) / 256;
  int64_t cap = (int64_t)p->sm_count * 8;
  grid = (int)(g < cap ? g : cap);
  return RAMP_OK;
}

static RecKey rec_key(const RampPlan* p, int det_comp, int64_t n, int32_t num_sim, int32_t seed,
                      const RampRng* rng) {
  RecKey k;
  memset(&k, 0, sizeof(k));
  k.det = det_comp; k.n = n; k.num_sim = num_sim; k.seed = seed;
  k.mode = rng ? rng->mode : 0;
  k.run_seed = rng ? rng->run_seed : 0u;
  k.tid_base = rng ? rng->tid_base : 0u;
  k.version = p->param_version;
  return k;
}

int ramp_forward_record(RampPlan* p, int32_t det_comp, int64_t n, int32_t num_sim, int32_t seed,
                        const RampRng* rng, void* stream) {
  if (!p || n < 0 || (rng && rng->seed_dev)) {
    set_err("ramp_forward_record: bad arguments (a device seed is not supported)");
    return RAMP_E_INVALID;
  }
  if (int rc0 = check_whole_chain(p, "ramp_forward_record")) return rc0;
  cudaStream_t s = (cudaStream_t)stream;
  SrcDev src;
  int rc = prep_adjoint(p, nullptr, 0, det_comp, nullptr, src, s);
  if (rc) return rc;
  AdjointArgs a;
  int grid;
  rc = adjoint_args(p, src, 0, n, num_sim, seed, rng, 0, nullptr, a, grid);
  if (rc) return rc;
  CK(launch_adjoint(a, grid, 1 | 4, s));
  p->rec = rec_key(p, det_comp, n, num_sim, seed, rng);
  p->rec_valid = true;
  return RAMP_OK;
}

int ramp_adjoint(RampPlan* p, const RampDiffParam* params, int n_params, int det_comp,
                 const float* dL_dH, int64_t n, int32_t num_sim, int32_t seed,
                 const RampRng* rng, int lr, double* grad, void* stream) {
  if (!p || !params || n_params <= 0 || n_params > RAMP_MAX_DIFF_PARAMS || !dL_dH || !grad ||
      n < 0) {
    set_err("ramp_adjoint: bad arguments");
    return RAMP_E_INVALID;
  }
  if (int rc0 = check_whole_chain(p, "ramp_adjoint")) return rc0;
  cudaStream_t s = (cudaStream_t)stream;
  SrcDev src;
  int rc = prep_adjoint(p, params, n_params, det_comp, dL_dH, src, s);
  if (rc) return rc;
  AdjointArgs a;
  int grid;
  rc = adjoint_args(p, src, n_params, n, num_sim, seed, rng, lr, grad, a, grid);
  if (rc) return rc;
  const RecKey k = rec_key(p, det_comp, n, num_sim, seed, rng);
  const bool reuse = p->rec_valid && !(rng && rng->seed_dev) && memcmp(&k, &p->rec, sizeof(k)) == 0;
  CK(launch_adjoint(a, grid, reuse ? 2 : (1 | 2), s));
  return RAMP_OK;
}

int ramp_seed_advance(int32_t* seed_dev, void* stream) {
  if (!seed_dev) { set_err("ramp_seed_advance: NULL seed"); return RAMP_E_INVALID; }
  CK(launch_seed_advance(seed_dev, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_debug_threefry(const uint32_t* c0, const uint32_t* tid, uint32_t* out, int64_t n,
                        void* stream) {
  if (!c0 || !tid || !out || n < 0) { set_err("bad arguments"); return RAMP_E_INVALID; }
  CK(launch_debug_threefry(c0, tid, out, n, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_debug_math(int fn, const float* a, const float* b, float* out, int64_t n,
                    void* stream) {
  if (!a || !out || n < 0) { set_err("bad arguments"); return RAMP_E_INVALID; }
  CK(launch_debug_math(fn, a, b, out, n, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_debug_rng_peak(int64_t n_threads, int32_t iters, uint32_t* out, void* stream) {
  if (!out || n_threads < 0 || iters < 0) { set_err("bad arguments"); return RAMP_E_INVALID; }
  CK(launch_debug_rng_peak(n_threads, iters, out, (cudaStream_t)stream));
  return RAMP_OK;
}

static bool pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

int ramp_debug_l2_peak(const float* buf, int64_t len, int64_t n_threads, int32_t iters,
                       float* out, void* stream) {
  if (!buf || !out || len % 4 != 0 || !pow2(len / 4) || n_threads < 0 || n_threads % 256 ||
      n_threads / 256 > INT32_MAX || iters < 0 || iters % 2 || ((uintptr_t)buf & 15)) {
    set_err("ramp_debug_l2_peak: buf 16-byte aligned, len/4 a power of two, n_threads a "
            "multiple of 256, iters even");
    return RAMP_E_INVALID;
  }
  CK(launch_debug_l2_peak((const float4*)buf, len / 4, n_threads, iters, out,
                          (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_debug_atomic_peak(float* bins, int64_t n_bins, int64_t n_threads, int32_t iters,
                           void* stream) {
  if (!bins || !pow2(n_bins) || n_bins > ((int64_t)1 << 31) || n_threads < 0 ||
      n_threads % 256 || n_threads / 256 > INT32_MAX || n_threads > UINT32_MAX || iters < 0) {
    set_err("ramp_debug_atomic_peak: n_bins a power of two, n_threads a multiple of 256");
    return RAMP_E_INVALID;
  }
  CK(launch_debug_atomic_peak(bins, n_bins, n_threads, iters, (cudaStream_t)stream));
  return RAMP_OK;
}

int ramp_chopper_run(const RampComp* comps, int n_comps, const RampBlock* blocks, int n_blocks,
                     int k) {
  return chopper_run(comps, n_comps, blocks, n_blocks, k);
}

int ramp_debug_chopper_cull(const RampComp* comps, int n_comps, const RampBlock* blocks,
                            int n_blocks, int k, const float* records, int64_t n, uint8_t* out) {
  if (!comps || n_comps <= 0 || n < 0 || (n > 0 && (!records || !out))) {
    set_err("ramp_debug_chopper_cull: bad arguments");
    return RAMP_E_INVALID;
  }
  const int nl = chopper_run(comps, n_comps, blocks, n_blocks, k);
  if (nl == 0) {
    set_err("ramp_debug_chopper_cull: no chopper run at component %d", k);
    return RAMP_E_INVALID;
  }
  /* the descriptor fields the bound reads, as make_comp sets them */
  std::vector<CompDev> d((size_t)n_comps);
  for (int j = 0; j < n_comps; ++j) {
    CompDev& q = d[(size_t)j];
    memset(&q, 0, sizeof(q));
    q.geom = comps[j].geom; q.scat = comps[j].scat;
    memcpy(q.pos, comps[j].pos, sizeof(q.pos));
    memcpy(q.gp, comps[j].gp, sizeof(q.gp));
    memcpy(q.sp, comps[j].sp, sizeof(q.sp));
    memcpy(q.si, comps[j].si, sizeof(q.si));
    if (comps[j].scat == RAMP_S_CHOPPER && (uint32_t)comps[j].si[0] != 0u)
      chopper_aux(comps[j], q.aux);
  }
  for (int64_t i = 0; i < n; ++i) {
    const float* r = records + 16 * i;
    out[i] = chopper_run_blocks(d.data(), k, nl, r[0], r[1], r[2], r[3], r[4], r[5], r[10]) ? 1 : 0;
  }
  return RAMP_OK;
}

int ramp_debug_speed_cull(const RampComp* comps, int n_comps, const RampBlock* blocks,
                          int n_blocks, int k, const float* source_p, const uint32_t* words,
                          int64_t n, uint8_t* out, int64_t* table_check) {
  if (!comps || n_comps <= 0 || !source_p || n < 0 || (n > 0 && (!words || !out))) {
    set_err("ramp_debug_speed_cull: bad arguments");
    return RAMP_E_INVALID;
  }
  const int nl = chopper_run(comps, n_comps, blocks, n_blocks, k);
  if (nl == 0) {
    set_err("ramp_debug_speed_cull: no chopper run at component %d", k);
    return RAMP_E_INVALID;
  }
  std::vector<CompDev> d((size_t)n_comps);
  for (int j = 0; j < n_comps; ++j) {
    CompDev& q = d[(size_t)j];
    memset(&q, 0, sizeof(q));
    q.geom = comps[j].geom; q.scat = comps[j].scat;
    memcpy(q.pos, comps[j].pos, sizeof(q.pos));
    memcpy(q.gp, comps[j].gp, sizeof(q.gp));
    memcpy(q.sp, comps[j].sp, sizeof(q.sp));
    memcpy(q.si, comps[j].si, sizeof(q.si));
    if (comps[j].scat == RAMP_S_CHOPPER && (uint32_t)comps[j].si[0] != 0u)
      chopper_aux(comps[j], q.aux);
  }
  std::unique_ptr<SpeedTab> T(new SpeedTab);
  SpeedRun& run = T->run;
  speed_run_prepare(d.data(), k, nl, source_p[0], source_p[1], source_p[2], source_p[3],
                    source_p[4], &run);
  const float e0 = source_p[5], de = source_p[6] - source_p[5];
  /* the choppers ordered as the device orders them, by how many of a
     sample of speeds (here those of the first 256 words) each one blocks */
  int blocked[SPEED_RUN_MAX] = {0};
  for (int64_t i = 0; i < n && i < 256; ++i) {
    const float iv = speed_iv_of_word(words[i], e0, de);
    for (int q = 0; q < run.n; ++q)
      if (iv > 0.0f && iv < 1e30f && speed_chopper_blocks(run, q, iv)) ++blocked[q];
  }
  speed_run_sort(&run, blocked);
  /* the device's speed table */
  speed_tab_range(T.get(), e0, de);
  for (int c = 0; c < T->ncell; ++c) {
    float lo, hi;
    speed_word_cell(c, e0, de, &lo, &hi);
    T->cell[c] = (uint8_t)speed_cell_verdict(run, lo, hi);
  }
  int64_t nd = 0, nm = 0;
  for (int64_t i = 0; i < n; ++i) {
    const bool by_table = speed_tab_blocks(*T, words[i]);
    const bool by_run = speed_run_blocks(run, speed_iv_of_word(words[i], e0, de));
    out[i] = by_table ? 1 : 0;
    nm += by_table != by_run;
    if (T->ncell > 0 &&
        T->cell[(words[i] >> SPEED_CELL_SHIFT) & (SPEED_CELLS - 1)] != SPEED_MIXED)
      ++nd;
  }
  if (table_check) {
    table_check[0] = nd;
    table_check[1] = nm;
  }
  return RAMP_OK;
}

}  // extern "C"

/* ======================================================================
 * ramp_trace_batched_noalloc — the batched fused path for callers that
 * must not allocate device memory while they trace: a host loop that runs
 * under a strict device-memory budget, or one whose device memory comes
 * from an external pool that forbids further allocation.  It uses only
 * memory that already exists.
 *
 * The per-call scratch of the one-launch batched kernel (the device copies
 * of every variant's component descriptors, the variant table and the
 * per-variant work-queue counters) lives in the file-scope array below
 * instead of plan-owned buffers that grow with cudaMalloc.  Its size is
 * fixed: RAMP_NOALLOC_MAX_VARIANTS variants and RAMP_NOALLOC_MAX_DESCS
 * component descriptors in total (variants x components), about 2.5 MB,
 * held by every GPU on which the library is loaded until the process
 * exits.  Tables (S(q,w), powder lines, mesh BVHs) must be ones the plan
 * already holds: a variant whose tables differ from every table the plan
 * uploaded is rejected.  Device status flags and dropped tally writes go to
 * the plan's own status word (allocated with the plan), so
 * ramp_plan_status reports them as for every other entry point.
 *
 * The first call on a device looks up the device address of the array
 * (cudaGetSymbolAddress, with that device current) and caches it; make that
 * first call before any stream capture.  All calls share the array, which
 * keeps the previous call's contents: each call overwrites the descriptors
 * and clears the counters before its launch, so two calls whose kernels
 * overlap on the GPU (different streams, no ordering) race and give wrong
 * results; order such calls on one stream.
 * ==================================================================== */
#define RAMP_NOALLOC_MAX_VARIANTS 256
#define RAMP_NOALLOC_MAX_DESCS 4096

struct NoallocLayout {
  VariantDev variants[RAMP_NOALLOC_MAX_VARIANTS];
  CompDev descs[RAMP_NOALLOC_MAX_DESCS];
  unsigned long long counters[2 * RAMP_NOALLOC_MAX_VARIANTS];   /* per-variant work queues */
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoallocLayout)];

#define RAMP_NOALLOC_MAX_DEVICES 64
static NoallocLayout* g_noalloc_dev[RAMP_NOALLOC_MAX_DEVICES];
/* host staging of the descriptor and variant tables (pageable copies
 * complete before cudaMemcpyAsync returns, so one buffer serves all calls) */
static NoallocLayout g_noalloc_host;
static std::mutex g_noalloc_mutex;

/* table lookup that never uploads */
static int lookup_table(RampPlan* p, const float* host, int64_t len, const float** dev,
                        HashMemo* memo) {
  static const float zero = 0.0f;
  if (len <= 0 || !host) { host = &zero; len = 1; }
  TabKey key(0, len, table_hash(host, len * (int64_t)sizeof(float), memo));
  auto it = p->tabs.find(key);
  if (it == p->tabs.end()) return RAMP_E_INVALID;
  *dev = (const float*)it->second.first;
  return RAMP_OK;
}

static int lookup_bvh(RampPlan* p, const float* pts, int64_t len, const float4** nodes_dev,
                      const float4** tris_dev, HashMemo* memo) {
  TabKey key(1, len, table_hash(pts, len * (int64_t)sizeof(float), memo));
  auto it = p->tabs.find(key);
  if (it == p->tabs.end()) {
    set_err("the mesh of a component is not held by the plan");
    return RAMP_E_INVALID;
  }
  *nodes_dev = (const float4*)it->second.first;
  *tris_dev = (const float4*)it->second.second;
  return RAMP_OK;
}

extern "C" int ramp_trace_batched_noalloc(RampPlan* p, const RampVariant* variants, int n_variants,
                                          const RampRng* rng, const RampTune* tune, void* stream) {
  if (!p || !variants || n_variants <= 0) {
    set_err("ramp_trace_batched_noalloc: bad arguments");
    return RAMP_E_INVALID;
  }
  if (int rc0 = check_whole_chain(p, "ramp_trace_batched_noalloc")) return rc0;
  const int nc = (int)p->comps.size();
  if (nc > RAMP_MAX_COMPS) {
    set_err("ramp_trace_batched_noalloc: at most %d components", RAMP_MAX_COMPS);
    return RAMP_E_RANGE;
  }
  if (n_variants > RAMP_NOALLOC_MAX_VARIANTS || (int64_t)n_variants * nc > RAMP_NOALLOC_MAX_DESCS) {
    set_err("ramp_trace_batched_noalloc: %d variants x %d components exceed the fixed scratch "
            "(at most %d variants and %d descriptors)", n_variants, nc,
            RAMP_NOALLOC_MAX_VARIANTS, RAMP_NOALLOC_MAX_DESCS);
    return RAMP_E_RANGE;
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= RAMP_NOALLOC_MAX_DEVICES) {
    set_err("ramp_trace_batched_noalloc: device %d beyond %d", dev, RAMP_NOALLOC_MAX_DEVICES);
    return RAMP_E_RANGE;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_dev[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      set_err("ramp_trace_batched_noalloc: cudaGetSymbolAddress failed: %s",
              cudaGetErrorString(e));
      return RAMP_E_CUDA;
    }
    g_noalloc_dev[dev] = (NoallocLayout*)ptr;
  }
  NoallocLayout* D = g_noalloc_dev[dev];
  NoallocLayout& H = g_noalloc_host;
  int block, grid;
  int64_t task;
  int32_t minb;
  tune_defaults(p, tune, block, grid, task, minb);
  int64_t n_max = 0;
  HashMemo memo;
  for (int v = 0; v < n_variants; ++v) {
    const RampVariant& V = variants[v];
    if (!V.comps || V.n < 0) {
      set_err("ramp_trace_batched_noalloc: variant %d: missing components", v);
      return RAMP_E_INVALID;
    }
    for (int j = 0; j < nc; ++j) {
      const RampComp& c = V.comps[j];
      if (c.geom != p->comps_in[j].geom || c.scat != p->comps_in[j].scat) {
        set_err("ramp_trace_batched_noalloc: variant %d component %d: kinds differ from the "
                "plan", v, j);
        return RAMP_E_INVALID;
      }
      int rc = validate_comp(c, j);
      if (!rc) rc = make_comp(p, c, H.descs[(size_t)v * nc + j], &memo, false);
      if (rc) return rc;
    }
    int rc = make_src(p, V.source, H.variants[v].src, false, &memo);
    if (rc) return rc;
    H.variants[v].n = V.n;
    H.variants[v].num_sim = V.num_sim;
    H.variants[v].seed = V.seed;
    H.variants[v].comps = D->descs + (size_t)v * nc;
    H.variants[v].item_off = 0;
    if (V.n > n_max) n_max = V.n;
  }
  if (n_max == 0) return RAMP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(D->descs, H.descs, (size_t)n_variants * nc * sizeof(CompDev),
                     cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(D->variants, H.variants, (size_t)n_variants * sizeof(VariantDev),
                     cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(D->counters, 0, 2 * (size_t)n_variants * sizeof(unsigned long long), s));
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.minb = minb;
  a.variants = D->variants;
  a.n_variants = n_variants;
  a.blocks = p->blocks_dev;
  a.n_blocks = (int32_t)p->blocks.size();
  a.n_comps = nc;
  a.rng.mode = rng ? rng->mode : 1;
  a.rng.run_seed = rng ? rng->run_seed : 0u;
  a.rng.one = 1u;
  a.rng.tid_base = 0u;
  a.st = p->status;             /* allocated with the plan: read by ramp_plan_status */
  a.workq = D->counters;
  a.workq_b = D->counters + n_variants;
  bool ext = p->ext;
  for (int v = 0; v < n_variants; ++v)
    if (ext_source(variants[v].source)) ext = true;
  a.ext = kind_set(ext, p->mesh);
  /* no survivor split here: it would need a buffer sized by the call */
  CK(launch_fused(a, block, batched_grid(n_max, grid), s));
  return RAMP_OK;
}
