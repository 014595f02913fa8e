/*
 * ramp.h — C ABI of libramp_cuda.so, the GB300 (sm_103a) implementation of
 * RAMP's per-neutron ray-tracing chain (moderator -> geometry -> scatter ->
 * detector tally).
 *
 * The reference (gcassella/RAMP) has no C ABI: its boundary is the Python
 * plugin API (mcramp/mcramp.py and the moderator/, geom/, scat/ classes),
 * which enqueues one OpenCL kernel per plugin call through pyopencl.  Each
 * entry point below names the reference call sequence it replaces.
 *
 * Conventions
 *   - every function returns 0 on success and a negative RAMP_E* code on
 *     failure; ramp_last_error() gives a message.  Nothing exits or traps.
 *   - all neutron state and all tallies are caller-owned device memory
 *     (plain pointers + sizes); a plan owns only the tables it uploads and a
 *     small status block.
 *   - plans are immutable after creation except for ramp_plan_set_*;
 *     concurrent calls on different streams with distinct state/tallies are
 *     safe, calls on one plan that share tallies race like the reference's
 *     float atomics do.
 *   - streams are passed as void* (a cudaStream_t; NULL = legacy default).
 */
#ifndef RAMP_H
#define RAMP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAMP_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define RAMP_OK              0
#define RAMP_E_INVALID      -1   /* bad argument or descriptor            */
#define RAMP_E_CUDA         -2   /* a CUDA runtime call failed            */
#define RAMP_E_NOMEM        -3   /* device allocation failed              */
#define RAMP_E_DEVICE       -4   /* a kernel raised a device status flag  */
#define RAMP_E_UNSUPPORTED  -5   /* component kind not available here     */
#define RAMP_E_RANGE        -6   /* size beyond a documented maximum      */

/* ---- device status flags (bit set in the plan's status word) ----------- */
#define RAMP_F_GUIDE_CAP      1u  /* guide bounce loop hit its hard cap     */
#define RAMP_F_POWDER_CAP     2u  /* powder line walk hit its hard cap      */
#define RAMP_F_TALLY_OOB      4u  /* a bin index fell outside its buffer    */
#define RAMP_F_BVH_STACK      8u  /* BVH traversal stack overflow           */
#define RAMP_F_WORKQ         16u  /* persistent work queue gave up          */

/* ---- neutron record lanes (NOTES:3-14, mcramp/include/consts.h:91-108) - */
enum RampLane {
  RAMP_X = 0, RAMP_Y, RAMP_Z, RAMP_VX, RAMP_VY, RAMP_VZ,
  RAMP_PX, RAMP_PY, RAMP_PZ, RAMP_P, RAMP_TOF,
  RAMP_MC,        /* sb: RNG draw counter, a float (rand.h:5,18)          */
  RAMP_PREVCOMP,  /* sc                                                   */
  RAMP_SD,        /* sd: Q of the last isotropic scatter                  */
  RAMP_SE,        /* se: omega (isotropic) / counted flag (counter)       */
  RAMP_DIE,       /* sf: termination flag                                 */
  RAMP_NLANES
};

/* ---- component kinds --------------------------------------------------- */
enum RampSourceKind {
  RAMP_SRC_FLAT = 1,   /* MFlat  moderator/flat_mod.py:10, flat_mod.cl:4  */
  RAMP_SRC_CONT = 2,   /* MCont  moderator/cont_mod.py:10, cont_mod.cl:11 */
  RAMP_SRC_ISIS = 3    /* MISIS  moderator/isis_mod.py:10, isis_mod.cl:15 */
};

enum RampGeomKind {
  RAMP_G_PLANE      = 1,  /* GPlane       geom/plane.cl:3               */
  RAMP_G_CYL_EXT    = 2,  /* GCylinderExt geom/cylinder_ext.cl:3        */
  RAMP_G_BANANA     = 3,  /* GBanana      geom/banana.cl:3              */
  RAMP_G_SPHERE     = 4,  /* GSphere      geom/sphere.cl:3              */
  RAMP_G_SPHERE_INT = 5,  /* GSphereInt   geom/sphere_int.cl:3          */
  RAMP_G_BOX        = 6,  /* GBox         geom/box.cl:3                 */
  RAMP_G_ARM        = 7,  /* GArm         geom/arm.cl:3                 */
  RAMP_G_MESH       = 8   /* GMesh        geom/mesh.cl:3 (BVH on GPU)   */
};

enum RampScatKind {
  RAMP_S_ARM       = 1,   /* SArm         scat/arm.cl:3                 */
  RAMP_S_GUIDE     = 2,   /* SGuide       scat/guide.cl:9               */
  RAMP_S_CHOPPER   = 3,   /* SChopper     scat/chopper.cl:4             */
  RAMP_S_ISOTROPIC = 4,   /* SIsotropic   scat/isotropic.cl:75          */
  RAMP_S_POWDERN   = 5,   /* SPowderN     scat/powderN.cl:5             */
  RAMP_S_DET1D     = 6,   /* SDetector1D  scat/detector1D.cl:20         */
  RAMP_S_DET2D     = 7,   /* SDetector2D  scat/detector2D.cl:31         */
  RAMP_S_COUNTER   = 8,   /* SCounter     scat/counter.cl:18            */
  RAMP_S_BEAMSTOP  = 9,   /* SBeamstop    scat/beamstop.cl:3            */
  RAMP_S_ATTENUATE = 10,  /* SAttenuate   no reference counterpart: Beer-
                             Lambert weight over the summed mesh chords */
  RAMP_S_MONO      = 11,  /* SMonochromator scat/monochromator.cl:22    */
  RAMP_S_POWDER1   = 12,  /* SPowder1     scat/powder1.cl:5             */
  RAMP_S_RESCAL    = 13,  /* SRescal      scat/rescal.cl:5: writes one
                             8-float event per neutron index into the
                             buffer bound by ramp_plan_set_buffer; plain
                             path, linear blocks only                   */
  RAMP_S_HOST      = 14   /* scattering done by the host between
                             ramp_component_enter and _leave (SMCPLOut
                             scat/mcpl_out.py:85, SMCPLIn mcpl_in.py:39);
                             plain path, linear blocks only             */
};

/* ---- descriptors ------------------------------------------------------- */
#define RAMP_NGP 12
#define RAMP_NSP 24
#define RAMP_NGI 4
#define RAMP_NSI 12
#define RAMP_NTAB 12

/* One moderator (the component with "source": true, mcramp.py:58-63).
 * p[]: mod_dim.x, mod_dim.y, target_dim.x, target_dim.y, target_dist,
 *      E_min, E_max, T1, I1, T2, I2, T3, I3, str_area, total
 * MISIS tables (host arrays, copied at plan creation): table[0] the flux
 * CDF over (energy row, time bin), (n_e - 1) * n_t values; table[1] the
 * n_t time bins (s); table[2] the n_e energy bin edges (meV); table[3] the
 * n_e cumulative flux at the energy edges (isis_mod.py:85-165).          */
typedef struct RampSource {
  int32_t kind;
  int32_t reserved;
  float p[16];
  const float* table[4];
  int64_t table_len[4];
} RampSource;

/* One non-source component (mcramp.py:65-108): a geometry kernel and a
 * scattering kernel sharing a frame (position, rotation) and an index.
 * Parameter slots per kind are listed in the Python plugin classes
 * (ramp_gb300/geom, ramp_gb300/scat) that fill them.                      */
typedef struct RampComp {
  int32_t geom;                 /* RampGeomKind                          */
  int32_t scat;                 /* RampScatKind                          */
  uint32_t idx;                 /* component index (mcramp.py:86,112)    */
  uint32_t restore;             /* component restore_neutron (:68,104)   */
  float pos[3];                 /* position (after "relative")           */
  float rot[3];                 /* Euler angles x,y,z in radians         */
  float gp[RAMP_NGP];           /* geometry float parameters             */
  float sp[RAMP_NSP];           /* scatter float parameters              */
  int32_t gi[RAMP_NGI];         /* geometry integer parameters           */
  int32_t si[RAMP_NSI];         /* scatter integer parameters            */
  const float* table[RAMP_NTAB];/* host tables, copied at plan creation  */
  int64_t table_len[RAMP_NTAB]; /* lengths in floats                     */
  float* tally;                 /* caller-owned tally (device memory)    */
  float* tally_err;             /* caller-owned sum of squared weights   */
  int64_t tally_len;            /* floats in each of tally / tally_err   */
} RampComp;

/* An execution block (mcramp.py:35-116, 368-382): components
 * [first, first+count) run linearly, or "multi" events non-linearly.     */
typedef struct RampBlock {
  int32_t first;
  int32_t count;
  int32_t linear;
  int32_t multi;
} RampBlock;

/* Neutron state in HBM, structure of arrays: lane l of neutron i lives at
 * soa[l*stride + i] (l < RAMP_NLANES); iidx[i] is the intersected-component
 * index buffer (doc/writing/buffers.rst:84-88).  stride is a multiple of 4
 * and soa is 16-byte aligned.                                             */
typedef struct RampState {
  float* soa;
  uint32_t* iidx;
  int64_t stride;
} RampState;

/* RNG keying.  mode 0 reproduces the reference stream exactly
 * (mcramp/include/rand.h:4-21): key = {tid, 0xdecafbad, 0xfacebead,
 * 0x12345678}, counter word 0 = (uint)sb, one Threefry-4x32-20 block per
 * draw, word x only.  mode 1 ("native") uses all four words of each block:
 * key = {tid, variant, run_seed, 0x12345678}, counter = {draw/4, ...}.  */
typedef struct RampRng {
  int32_t mode;
  uint32_t run_seed;
  uint32_t tid_base;   /* global index of neutron 0 of this call: a rank
                          tracing indices [tid_base, tid_base+n) of a
                          sharded chunk keys its neutrons exactly as a
                          single-device run would                         */
  uint32_t reserved;
  const int32_t* seed_dev;  /* optional (device): when set, the chunk seed
                          is read here when the kernel runs instead of the
                          seed argument — what lets a CUDA graph replay
                          draw a new seed each time (ramp_seed_advance)   */
} RampRng;

/* One variant of a batched fused launch: its own components (same kinds
 * and count as the plan's, different parameters and tallies), its own
 * neutron count, chunk weight normalisation and per-chunk seed.           */
typedef struct RampVariant {
  const RampComp* comps;        /* n_comps entries (host memory)         */
  RampSource source;            /* the variant's moderator               */
  int64_t n;                    /* histories in this variant             */
  int32_t num_sim;              /* p = 1/num_sim (flat_mod.cl:26)        */
  int32_t seed;                 /* randint(0,4096) stand-in              */
} RampVariant;

/* Launch configuration of the whole-chain kernels, chosen by the
 * autotuner (ramp_gb300/autotune.py); 0 = default.                        */
typedef struct RampTune {
  int32_t block;                /* threads per CTA: 256 (0) or 128 (the
                                   whole-chain kernels are compiled for at
                                   most 256); blocks_per_sm counts CTAs
                                   of this size                          */
  int32_t blocks_per_sm;        /* persistent CTAs per SM (register cap:
                                   3 or 4; 0: 4)                         */
  int32_t chunk;                /* neutrons per span; sizes the grid of a
                                   single-instrument launch (0: about
                                   eight spans per resident CTA)        */
  int32_t privatize;            /* ramp_trace_fused without split or walk:
                                   1 = detectors (SDetector1D/2D) whose two
                                   histograms fit, in chain order, in 48 KB
                                   of shared memory are accumulated per
                                   CTA there and merged into global memory
                                   as the CTA ends (0: warp-aggregated
                                   atomics into L2, the only choice for
                                   larger histograms)                   */
  int32_t split;                /* fused path: split the chain before this
                                   component (0: off; not inside a
                                   non-linear block).  Stage A appends the
                                   neutrons alive there to a survivor
                                   buffer in HBM (96 B per history of the
                                   launch, owned by the plan unless the
                                   caller sets one with
                                   ramp_plan_set_survivors) and stage B
                                   traces them 32 to a warp.  Ignored by
                                   ramp_trace_batched_noalloc.           */
  int32_t streams;              /* ramp_trace_batched: 0 or 1 = one
                                   launch (or, split, two) whose grid row
                                   v traces variant v; n >= 2: each
                                   variant is a launch of its own, on up
                                   to n concurrent streams (at most 16).
                                   Either way each variant has its own
                                   work counters and its own range of
                                   the survivor buffer.                  */
  int32_t walk;                 /* fused path, chains without the
                                   extended kinds: 1 = split before the
                                   first GMesh component of a linear
                                   block (replacing `split`); the second
                                   kernel walks the mesh hierarchy one
                                   node per pass on each lane and a lane
                                   whose walk is over takes the next
                                   waiting neutron (buffer as for
                                   `split`).  Ignored without such a
                                   component.                            */
  int32_t cull;                 /* fused path, runs without carry
                                   buffers: 1 = split before component
                                   `split` (which may then be 0: stage A
                                   runs the moderator alone) and let
                                   stage A also retire every neutron that
                                   certainly cannot pass the disk
                                   choppers (or misses a guide) of the
                                   run of on-axis straight guides and
                                   choppers starting there
                                   (ramp_chopper_run); only tallies are
                                   observable, and those neutrons would
                                   add nothing to them.  RAMP_E_INVALID
                                   without such a run.  Not with `walk`
                                   or in the one-launch batched layout of
                                   chains with the extended kinds.       */
} RampTune;

typedef struct RampPlan RampPlan;

/* ---- API --------------------------------------------------------------- */

int ramp_version(void);

/* Host-readable message for the last failing call on this thread.        */
int ramp_last_error(char* buf, int len);

/* Validate descriptors, precompute frame rotations, upload tables (and a
 * BVH for meshes).  Replaces the per-plugin constructors that build
 * OpenCL programs and buffers (mcramp.py:45-116, e.g. plane.py:63-73,
 * isotropic.py:41-155, powderN.py:50-77, mesh.py:60-81).                 */
int ramp_plan_create(const RampSource* source, const RampComp* comps,
                     int n_comps, const RampBlock* blocks, int n_blocks,
                     RampPlan** out);
int ramp_plan_destroy(RampPlan* plan);

/* Run linear components [k0, k1) over neutrons [0, n) (each a k_linear
 * pass): the pieces of a linear block around a host component.          */
int ramp_run_components(RampPlan* plan, int32_t k0, int32_t k1, const RampState* st,
                        int64_t n, const RampRng* rng, void* stream);

/* The device halves of a host component's pass (mcramp.py:124-157):
 * enter = frame transform, intersection, termination; leave = inverse
 * transform.  The host acts on the state in between.                    */
int ramp_component_enter(RampPlan* plan, int32_t comp, const RampState* st, int64_t n,
                         const RampRng* rng, void* stream);
int ramp_component_leave(RampPlan* plan, int32_t comp, const RampState* st, int64_t n,
                         void* stream);

/* Order-preserving compaction of neutrons [0, n) whose die lane is not
 * exactly 1 (mcpl_out.py:103): row r of out holds the lanes set in the
 * bit mask `lanes` (ascending lane order) of the r-th such neutron; *count
 * (device) receives the number of rows.  out holds n rows at most;
 * scratch holds ceil(n / 1024) int64.                                    */
int ramp_gather_alive(const RampState* st, int64_t n, uint32_t lanes, float* out,
                      int64_t* scratch, int64_t scratch_len, int64_t* count, void* stream);

/* Bind component comp's output buffer (device, len floats): the event
 * list of an SRescal component (8 floats per neutron index of a chunk).
 * Replaces the buffer the descriptor named at plan creation.            */
int ramp_plan_set_buffer(RampPlan* plan, int32_t comp, float* buf, int64_t len);

/* Allocate the plan's survivor buffer for split fused launches
 * (RampTune.split) of up to n histories now, e.g. before capturing them
 * in a CUDA graph (a split launch otherwise grows it on first use).    */
int ramp_plan_reserve(RampPlan* plan, int64_t n);

/* Read and clear the plan's device status flags (RAMP_F_*) and the count
 * of nonzero-weight tally writes that fell outside their buffers (a write
 * of weight zero loses nothing and is not counted).  Synchronises.       */
int ramp_plan_status(RampPlan* plan, uint32_t* flags, uint64_t* oob_drops);

/* Moderator pass over neutrons [0, n): replaces gen_prg
 * (flat_mod.py:24-32, cont_mod.py:137-152).  Every record is regenerated
 * and its counter seeded with seed + previous sb (flat_mod.cl:19).        */
int ramp_generate(RampPlan* plan, const RampState* st, int64_t n,
                  int32_t num_sim, int32_t seed, const RampRng* rng,
                  void* stream);

/* One execution block over neutrons [0, n): replaces
 * ExecutionBlock.execute (mcramp.py:118-220).  A linear block launches one
 * kernel per component (transform, intersect, terminate, scatter and
 * untransform fused); a non-linear block launches one kernel running all
 * its "multi" events.                                                     */
int ramp_run_block(RampPlan* plan, int block, const RampState* st,
                   int64_t n, const RampRng* rng, void* stream);

/* The plain path for one chunk: ramp_generate + ramp_run_block over every
 * block (one iteration of the chunk loop, mcramp.py:442-455).            */
int ramp_trace_plain(RampPlan* plan, const RampState* st, int64_t n,
                     int32_t num_sim, int32_t seed, const RampRng* rng,
                     void* stream);

/* The fused path for one chunk: the whole chain in one persistent kernel,
 * each neutron in registers from the moderator to its last component.
 * sb_carry / iidx_carry (optional, both NULL = all zero, i.e. a fresh
 * execute()) hold per index the final RNG counter and index-buffer value
 * of the previous chunk and receive this chunk's; they are what makes
 * multi-chunk runs reproduce the reference keying (flat_mod.cl:19) with
 * nothing else of the neutron state in memory.  Without carry buffers only
 * the tallies are observable, and a neutron whose weight becomes exactly
 * zero is retired at once (every later weight factor multiplies it and
 * every tally adds p or p^2, so it could only add zeros).               */
int ramp_trace_fused(RampPlan* plan, int64_t n, int32_t num_sim,
                     int32_t seed, const RampRng* rng, float* sb_carry,
                     uint32_t* iidx_carry, const RampTune* tune,
                     void* stream);

/* Batched fused path: n_variants instrument variants with uneven neutron
 * counts, by default in one launch whose grid row v traces variant v
 * (RampTune.streams >= 2: one launch per variant over that many streams).
 * Variant v's histories are keyed by its own index, count and seed, so
 * each variant's tallies are those of tracing it alone (no reference
 * counterpart: the reference runs one Instrument per execute()).          */
int ramp_trace_batched(RampPlan* plan, const RampVariant* variants,
                       int n_variants, const RampRng* rng,
                       const RampTune* tune, void* stream);

/* ---- differentiation ---------------------------------------------------
 * Parameters that enter neutron weights smoothly.  kind selects the
 * descriptor value, comp the component (index into the plan's components;
 * ignored for the source).  POWDER_SIGMA_ABS is the descriptor value
 * sigma_abs * v = pack * sigma_abs / vc * 100 (powderN.py:65).           */
#define RAMP_DP_GUIDE_R0          1
#define RAMP_DP_GUIDE_QC          2
#define RAMP_DP_GUIDE_ALPHA       3
#define RAMP_DP_GUIDE_M           4
#define RAMP_DP_GUIDE_W           5
#define RAMP_DP_SOURCE_T          6   /* T1 = T2 = T3 of MCont            */
#define RAMP_DP_POWDER_SIGMA_ABS  7
#define RAMP_MAX_DIFF_PARAMS     32

typedef struct RampDiffParam {
  int32_t kind;
  int32_t comp;
} RampDiffParam;

/* Set one parameter of a plan in place (no counterpart in the reference:
 * there, changing a parameter means building a new Instrument).          */
int ramp_plan_set_param(RampPlan* plan, int32_t kind, int32_t comp, float value);

/* Gradient of a loss of one detector's histogram with respect to
 * n_params parameters (no counterpart in the reference).  dL_dH is dL/dH
 * per bin of component det_comp's histogram (device memory).  The chain is
 * replayed for neutrons [0, n) with the chunk parameters of the forward
 * run (num_sim, seed, rng): the counter-based RNG recomputes every
 * neutron's state at every component boundary exactly.  Per neutron the
 * kernel accumulates d log p / d theta (analytic local derivatives of the
 * reflectivity, the Maxwellian weight and the powder attenuation, the
 * powder depth reparameterised through its inverse CDF) and, at each tally
 * by the loss detector, adds dL/dH_bin * p * d log p / d theta to grad
 * (device, double, n_params entries, accumulated).  lr = 1 adds the
 * likelihood-ratio terms of the powder's transmit/scatter branch (an
 * unbiased estimator; lr = 0 is the pathwise derivative that central
 * finite differences with common random numbers measure).  Only neutrons
 * the loss detector counts carry a term: a first pass lists them and only
 * they are replayed with derivatives; after ramp_forward_record with the
 * same detector, chunk parameters and parameter values, its list is used
 * and the first pass skipped.                                            */
int ramp_adjoint(RampPlan* plan, const RampDiffParam* params, int n_params,
                 int det_comp, const float* dL_dH, int64_t n, int32_t num_sim,
                 int32_t seed, const RampRng* rng, int lr, double* grad,
                 void* stream);

/* The forward histograms of a differentiable run (every tally of the
 * chain, as a fused launch of n neutrons with these chunk parameters
 * would add) together with the list of neutrons component det_comp
 * counts, kept in the plan for the next ramp_adjoint on the same run.
 * No counterpart in the reference.                                       */
int ramp_forward_record(RampPlan* plan, int32_t det_comp, int64_t n, int32_t num_sim,
                        int32_t seed, const RampRng* rng, void* stream);

/* ramp_trace_batched without device allocation.  No counterpart in the
 * reference.  For callers that may not allocate device memory while
 * tracing (a host loop under a fixed device-memory budget, or one whose
 * memory comes from an external pool that forbids further allocation):
 * the descriptor and variant tables and the per-variant work counters of
 * the one-launch batched kernel (a grid row per variant, no split) live in
 * one fixed file-scope device array (at most 256 variants and 4096
 * component descriptors, about 2.5 MB per GPU, held until exit) instead of
 * plan-owned buffers.  Every variant's tables must already be held by the
 * plan.  Status flags and dropped tally writes go to the plan's status
 * word, read by ramp_plan_status.  The first call on a device resolves the
 * array's address; make it before any stream capture.  Calls share the
 * array, so calls whose kernels overlap on the GPU race; order them on one
 * stream.  Sizes beyond the maximum return RAMP_E_RANGE.                  */
int ramp_trace_batched_noalloc(RampPlan* plan, const RampVariant* variants,
                               int n_variants, const RampRng* rng,
                               const RampTune* tune, void* stream);

/* Draw the next chunk seed on the device: seed_dev[0] receives a value in
 * [0, 4096] (the range of the per-chunk randint(0, 4096) seed,
 * flat_mod.py:32) from a 64-bit LCG whose state is seed_dev[2..3].  For
 * CUDA graphs: captured after a trace, every replay traces a new chunk.  */
int ramp_seed_advance(int32_t* seed_dev, void* stream);

/* Debug/test entry points: evaluate the device RNG and math on a vector
 * of inputs (used by the parity tests, not by the chain).                 */
int ramp_debug_threefry(const uint32_t* ctr0_dev, const uint32_t* tid_dev,
                        uint32_t* out_x_dev, int64_t n, void* stream);
int ramp_debug_math(int fn, const float* a_dev, const float* b_dev,
                    float* out_dev, int64_t n, void* stream);

/* Measurement kernel: n_threads threads each evaluate `iters` dependent
 * Threefry-4x32-20 blocks (two independent chains per thread) and xor the
 * results into out_dev[thread].  Its rate is the Threefry throughput ceiling
 * the fused kernel is compared against.                                   */
int ramp_debug_rng_peak(int64_t n_threads, int32_t iters, uint32_t* out_dev,
                        void* stream);

/* Measurement kernels for the rooflines: the L2 read bandwidth (n_threads
 * threads, a multiple of 256, each read `iters` (even) float4 of buf, len
 * floats with len/4 a power of two, through loads that bypass L1; out
 * receives n_threads floats) and the L2 float-atomic throughput (n_threads
 * threads each add 1 to `iters` bins of an n_bins histogram, n_bins a power
 * of two, a warp's lanes to one 128-byte line).                         */
int ramp_debug_l2_peak(const float* buf, int64_t len, int64_t n_threads, int32_t iters,
                       float* out, void* stream);
int ramp_debug_atomic_peak(float* bins, int64_t n_bins, int64_t n_threads, int32_t iters,
                           void* stream);

/* Host helper (no GPU): the hierarchy the plan builds for a GMesh over
 * pts[n_tri*9], walked for n_rays rays (6 floats each: position and
 * velocity in the mesh frame) as a walk that needs every crossing reads
 * it: out[0] inner nodes read (64 bytes each), out[1] triangles read (48
 * bytes each), out[2] rays meeting the mesh box.  The algorithmic L2
 * bytes of the mesh imaging roofline.                                   */
int ramp_bvh_walk_counts(const float* pts, int64_t n_tri, const float* rays, int64_t n_rays,
                         int64_t* out);

/* Bytes of the survivor buffer that a split fused launch (RampTune.split,
 * walk, cull) of n histories uses: 96 per history (a 72-byte record and,
 * after a mesh walk, its 24-byte result), rounded up to work items of 128
 * histories, plus 4 per work item.                                        */
int64_t ramp_survivor_bytes(int64_t n);

/* Let the plan's split launches keep their survivors in caller-owned
 * device memory (buf, 16-byte aligned, `bytes` long) instead of a buffer
 * the plan allocates; a launch that needs more than `bytes` uses the
 * plan's own.  buf NULL goes back to plan-owned buffers.  The memory must
 * stay valid while launches that use it run (a caching allocator keeps a
 * multi-gigabyte buffer from being allocated again for every new plan). */
int ramp_plan_set_survivors(RampPlan* p, void* buf, int64_t bytes);

/* Host helper (no GPU): the length of the chopper look-ahead run that
 * starts at component k (RampTune.cull), 0 when there is none.  The run:
 * components of the linear block holding k, each unrotated, centred on the
 * z axis (pos x = y = 0), with a z-normal GPlane and restore_neutron 0,
 * non-overlapping at non-decreasing z: straight SGuides (w1 = w2, h1 = h2)
 * and SChoppers in any order, up to the last chopper before the first
 * component that is neither; then, when the component right after that
 * chopper is an on-axis, unrotated GCylinderExt with restore_neutron 0
 * starting beyond it, that cylinder as the run's target (a neutron whose
 * line certainly misses its box dies there).  From a neutron's state
 * before such a run, the time and place it meets each component's plane
 * follow within tight bounds (vz does not change along it; the guides fold
 * the transverse motion at their walls).                                  */
int ramp_chopper_run(const RampComp* comps, int n_comps, const RampBlock* blocks, int n_blocks,
                     int k);

/* Host check (no GPU) of the look-ahead bound the device applies: for n
 * neutron records (16 floats each, stride 16: position, velocity, spin,
 * weight, time, ...; laboratory frame, before component k) out[i] = 1 when
 * the neutron certainly cannot pass a chopper of the run at k, else 0.
 * RAMP_E_INVALID when there is no run at k.                              */
int ramp_debug_chopper_cull(const RampComp* comps, int n_comps, const RampBlock* blocks,
                            int n_blocks, int k, const float* records, int64_t n, uint8_t* out);

/* Host check (no GPU) of the speed-only bound of the lean stage A: a flat
 * or MCont moderator with parameters source_p (moderator width and
 * height, target width and height, target distance, E_min, E_max:
 * RampSource.p[0..6]); out[i] = 1 when no neutron whose energy draw gave
 * the Threefry word words[i] can pass the choppers of the run at
 * component k (the run must start where the moderator's neutrons enter
 * the chain), else 0.  The answers come, as on the device, from a table
 * of cells of the word and, outside its decided cells, the per-chopper
 * test.  table_check (may be NULL): [0] the words a table cell decided,
 * [1] the words where the table's answer differs from the per-chopper
 * test's (0 unless the table is wrong).                                   */
int ramp_debug_speed_cull(const RampComp* comps, int n_comps, const RampBlock* blocks,
                          int n_blocks, int k, const float* source_p, const uint32_t* words,
                          int64_t n, uint8_t* out, int64_t* table_check);

#ifdef __cplusplus
}
#endif

#endif /* RAMP_H */
