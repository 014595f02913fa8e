/*
 * driver.cpp — TEST INFRASTRUCTURE ONLY.  Runs the reference's own OpenCL
 * kernels, compiled as host C++ through clshim.h, over one chunk of an
 * instrument, with the reference's sequencing (mcramp/mcramp.py:118-220):
 * the moderator's generate_neutrons, then for each component of a linear
 * block transform, the geometry kernel, terminate, the scattering kernel
 * and untransform, each as one pass over every work item; for non-linear
 * blocks "multi" rounds of (transform, geometry, untransform) over all
 * components followed by (transform, scattering, untransform).
 *
 * Its inputs are the descriptors the oracle takes (include/ramp.h: the
 * plugin classes of ramp_gb300 fill them from the instrument file), turned
 * back here into each kernel's argument list in the order of the kernel's
 * signature, as the reference plugins pass them (e.g. scat/guide.py:91-104,
 * geom/plane.py:49-57).  Buffers the reference reads or writes past their
 * ends (detector bins at the top edge, the powder line walk, the MISIS
 * table scans) are padded with zeros, so those accesses stay inside this
 * process's memory; tally writes that land in the padding are counted and
 * dropped, as the oracle does.
 *
 * Built by oracle/refcl/build.py into oracle/_ref/ (git-ignored), once with
 * the shared math library (REFCL_RMATH) and once with the C library's.
 */
#include "clshim.h"

#include <vector>
#include <omp.h>

#include "../../include/ramp.h"

thread_local uint refcl_gid;

/* the reference kernels, each file in a namespace of its own (several
 * define functions of the same name: generate_neutrons, intersect, arm,
 * detector, intersect_sphere, atomicAdd_g_f, rand) */
namespace k_flat {
REFCL_BUILTINS
#include "moderator/flat_mod.cl"
}
namespace k_cont {
REFCL_BUILTINS
#include "moderator/cont_mod.cl"
}
namespace k_isis {
REFCL_BUILTINS
#include "moderator/isis_mod.cl"
}
namespace k_frame {
REFCL_BUILTINS
#include "scat/frametransform.cl"
}
namespace k_term {
REFCL_BUILTINS
#include "scat/terminator.cl"
}
namespace k_plane {
REFCL_BUILTINS
#include "geom/plane.cl"
}
namespace k_cyl {
REFCL_BUILTINS
#include "geom/cylinder_ext.cl"
}
namespace k_banana {
REFCL_BUILTINS
#include "geom/banana.cl"
}
namespace k_sphere {
REFCL_BUILTINS
#include "geom/sphere.cl"
}
namespace k_sphere_int {
REFCL_BUILTINS
#include "geom/sphere_int.cl"
}
namespace k_box {
REFCL_BUILTINS
#include "geom/box.cl"
}
namespace k_garm {
REFCL_BUILTINS
#include "geom/arm.cl"
}
namespace k_mesh {
REFCL_BUILTINS
#include "geom/mesh.cl"
}
namespace k_sarm {
REFCL_BUILTINS
#include "scat/arm.cl"
}
namespace k_guide {
REFCL_BUILTINS
#include "scat/guide.cl"
}
namespace k_chopper {
REFCL_BUILTINS
#include "scat/chopper.cl"
}
namespace k_iso {
REFCL_BUILTINS
#include "scat/isotropic.cl"
}
namespace k_powdern {
REFCL_BUILTINS
#include "scat/powderN.cl"
}
namespace k_det1d {
REFCL_BUILTINS
#include "scat/detector1D.cl"
}
namespace k_det2d {
REFCL_BUILTINS
#include "scat/detector2D.cl"
}
namespace k_counter {
REFCL_BUILTINS
#include "scat/counter.cl"
}
namespace k_beamstop {
REFCL_BUILTINS
#include "scat/beamstop.cl"
}
namespace k_mono {
REFCL_BUILTINS
#include "scat/monochromator.cl"
}
namespace k_powder1 {
REFCL_BUILTINS
#include "scat/powder1.cl"
}
namespace k_rescal {
REFCL_BUILTINS
#include "scat/rescal.cl"
}

namespace {

/* one kernel launch: the work items [0, n) */
template <class F> void launch(int64_t n, F f) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    refcl_gid = (uint)i;
    f();
  }
}

/* a zero-padded copy of a host table: `front` zeros, the table, `back` zeros */
struct Padded {
  std::vector<float> buf;
  int64_t front = 0;
  Padded(const float* t, int64_t len, int64_t front_, int64_t back) : front(front_) {
    if (len < 0 || !t) len = 0;
    buf.assign((size_t)(front + len + back), 0.0f);
    if (len) memcpy(buf.data() + front, t, (size_t)len * sizeof(float));
  }
  float* p() { return buf.data() + front; }
};

/* a tally with zero padding behind it; in-range bins are copied back into
 * the caller's tally and nonzero padding writes are counted */
struct Tally {
  float* dst;
  int64_t len;
  std::vector<float> buf;
  Tally(float* d, int64_t l, int64_t pad) : dst(d), len(l) {
    buf.assign((size_t)(l + pad), 0.0f);
    if (d && l) memcpy(buf.data(), d, (size_t)l * sizeof(float));
  }
  float* p() { return buf.data(); }
  uint64_t finish() {
    if (dst && len) memcpy(dst, buf.data(), (size_t)len * sizeof(float));
    uint64_t drops = 0;
    for (size_t k = (size_t)len; k < buf.size(); ++k) drops += buf[k] != 0.0f;
    return drops;
  }
};

struct Run {
  float16* nb;
  float8* ib;
  uint* ii;
  int64_t n;
  uint64_t oob = 0;
};

inline float3 f3(const float* a) { return float3(a[0], a[1], a[2]); }

void transform(Run& r, const RampComp& c) {
  const float3 pos = f3(c.pos), rot = f3(c.rot);
  launch(r.n, [&] { k_frame::transform(r.nb, pos, rot); });
}

void untransform(Run& r, const RampComp& c) {
  const float3 pos = f3(c.pos), rot = f3(c.rot);
  launch(r.n, [&] { k_frame::untransform(r.nb, pos, rot); });
}

void terminate(Run& r, const RampComp& c) {
  launch(r.n, [&] { k_term::terminate(r.nb, r.ib, c.restore); });
}

int geometry(Run& r, const RampComp& c) {
  const uint idx = c.idx;
  switch (c.geom) {
    case RAMP_G_PLANE:
      launch(r.n, [&] { k_plane::intersect_plane(r.nb, r.ib, r.ii, idx, c.gp[0], c.gp[1],
                                                  (uint)c.gi[0]); });
      return 0;
    case RAMP_G_CYL_EXT:
      launch(r.n, [&] { k_cyl::intersect(r.nb, r.ib, r.ii, idx, c.gp[0], c.gp[1]); });
      return 0;
    case RAMP_G_BANANA:
      launch(r.n, [&] { k_banana::intersect_banana(r.nb, r.ib, r.ii, idx, c.gp[0], c.gp[1],
                                                    c.gp[2], c.gp[3]); });
      return 0;
    case RAMP_G_SPHERE:
      launch(r.n, [&] { k_sphere::intersect_sphere(r.nb, r.ib, r.ii, idx, c.gp[0]); });
      return 0;
    case RAMP_G_SPHERE_INT:
      launch(r.n, [&] { k_sphere_int::intersect_sphere(r.nb, r.ib, r.ii, idx, c.gp[0]); });
      return 0;
    case RAMP_G_BOX:
      launch(r.n, [&] { k_box::intersect_box(r.nb, r.ib, r.ii, idx, c.gp[0], c.gp[1],
                                              c.gp[2]); });
      return 0;
    case RAMP_G_ARM:
      launch(r.n, [&] { k_garm::arm(r.nb, r.ib, r.ii, idx); });
      return 0;
    case RAMP_G_MESH: {
      Padded pts(c.table[0], c.table_len[0], 0, 0);
      const uint ntri = (uint)(c.table_len[0] / 9);
      launch(r.n, [&] { k_mesh::intersect(r.nb, r.ib, r.ii, idx, pts.p(), ntri, c.gp[0],
                                          c.gp[1], c.gp[2], c.gp[3], c.gp[4], c.gp[5],
                                          (uint)c.gi[0]); });
      return 0;
    }
    default:
      return RAMP_E_UNSUPPORTED;
  }
}

int scatter(Run& r, const RampComp& c) {
  const uint idx = c.idx;
  switch (c.scat) {
    case RAMP_S_ARM:
      launch(r.n, [&] { k_sarm::arm(r.nb, r.ib, r.ii, idx); });
      return 0;
    case RAMP_S_BEAMSTOP:
      launch(r.n, [&] { k_beamstop::beamstop(r.nb, r.ib, r.ii, idx); });
      return 0;
    case RAMP_S_COUNTER: {
      Tally t(c.tally, c.tally_len, 0);
      launch(r.n, [&] { k_counter::counter(r.nb, r.ib, r.ii, idx, t.p()); });
      r.oob += t.finish();
      return 0;
    }
    case RAMP_S_GUIDE:
      launch(r.n, [&] { k_guide::guide_scatter(r.nb, r.ib, r.ii, idx, c.sp[0], c.sp[1], c.sp[2],
                                               c.sp[3], c.sp[4], c.sp[5], c.sp[6], c.sp[7],
                                               c.sp[8], c.sp[9], (uint)c.si[0]); });
      return 0;
    case RAMP_S_CHOPPER:
      launch(r.n, [&] { k_chopper::chopper(r.nb, r.ib, r.ii, idx, c.sp[0], c.sp[1], c.sp[2],
                                           (uint)c.si[0], c.sp[3], c.sp[4]); });
      return 0;
    case RAMP_S_ISOTROPIC: {
      /* per channel (coh, inc, mag): q, w, p(w) cdf, p(q|w) cdf; the cdf
         scans read one entry past a row at most (zero padding) */
      std::vector<Padded> t;
      t.reserve(12);
      for (int k = 0; k < 12; ++k) t.emplace_back(c.table[k], c.table_len[k], 0, 64);
      launch(r.n, [&] {
        k_iso::isotropic_scatter(
            r.nb, r.ib, r.ii, idx,
            t[0].p(), t[1].p(), t[2].p(), t[3].p(), (uint)c.si[1], (uint)c.si[2],
            c.sp[1], c.sp[2], c.sp[3],
            t[4].p(), t[5].p(), t[6].p(), t[7].p(), (uint)c.si[3], (uint)c.si[4],
            c.sp[4], c.sp[5], c.sp[6],
            t[8].p(), t[9].p(), t[10].p(), t[11].p(), (uint)c.si[5], (uint)c.si[6],
            c.sp[7], c.sp[8], c.sp[9],
            c.sp[0], (uint)c.si[0]);
      });
      return 0;
    }
    case RAMP_S_POWDERN: {
      /* The line walk (powderN.cl:77-85) reads past the last line when the
         rounded cumulative sum stays below the deviate.  The padding makes
         that read end the walk with the last line's q, which is the
         oracle's reading (walk stops at the last line): sigma past the end
         is +inf, q past the end repeats the last q. */
      const int64_t nl = c.si[0];
      Padded s2(c.table[0], c.table_len[0], 0, 64);
      Padded q(c.table[1], c.table_len[1], 0, 64);
      for (int64_t k = nl; k < nl + 64; ++k) {
        s2.p()[k] = __builtin_inff();
        q.p()[k] = nl > 0 ? q.p()[nl - 1] : 0.0f;
      }
      launch(r.n, [&] { k_powdern::powderN(r.nb, r.ib, r.ii, idx, s2.p(), c.sp[0], q.p(),
                                           c.sp[1], (uint)c.si[0], (uint)c.si[1]); });
      return 0;
    }
    case RAMP_S_DET1D: {
      Tally h(c.tally, c.tally_len, 8), e(c.tally_err, c.tally_len, 8);
      const float3 b(c.sp[0], c.sp[1], c.sp[2]);
      launch(r.n, [&] { k_det1d::detector(r.nb, r.ib, r.ii, idx, h.p(), e.p(), b, (uint)c.si[1],
                                          (uint)c.si[0]); });
      r.oob += h.finish();
      e.finish();
      return 0;
    }
    case RAMP_S_DET2D: {
      /* round() bins reach index n on each axis: flat index <= n1 n2 + n2 */
      const int64_t pad = 2 * (int64_t)c.si[3] + 8;
      Tally h(c.tally, c.tally_len, pad), e(c.tally_err, c.tally_len, pad);
      const float3 b1(c.sp[0], c.sp[1], c.sp[2]), b2(c.sp[3], c.sp[4], c.sp[5]);
      launch(r.n, [&] { k_det2d::detector(r.nb, r.ib, r.ii, idx, h.p(), e.p(), b1, b2,
                                          (uint)c.si[2], (uint)c.si[3], (uint)c.si[0],
                                          (uint)c.si[1], (uint)c.si[4]); });
      r.oob += h.finish();
      e.finish();
      return 0;
    }
    case RAMP_S_MONO: {
      Padded gx(c.table[0], c.table_len[0], 0, 0), gw(c.table[1], c.table_len[1], 0, 0);
      launch(r.n, [&] { k_mono::monochromator(r.nb, r.ib, r.ii, idx, c.sp[0], c.sp[1], c.sp[2],
                                              (uint)c.si[0], (uint)c.si[1], c.sp[3], c.sp[4],
                                              c.sp[5], c.sp[6], c.sp[7], c.sp[8], gx.p(),
                                              gw.p(), (uint)c.table_len[0]); });
      return 0;
    }
    case RAMP_S_POWDER1:
      launch(r.n, [&] { k_powder1::powder1(r.nb, r.ib, r.ii, idx, c.sp[0], c.sp[1], c.sp[2],
                                           c.sp[3]); });
      return 0;
    case RAMP_S_RESCAL: {
      if (!c.tally || c.tally_len < 8 * r.n) return RAMP_E_INVALID;
      const float3 tg(c.sp[0], c.sp[1], c.sp[2]);
      float8* ev = reinterpret_cast<float8*>(c.tally);
      launch(r.n, [&] { k_rescal::rescal(r.nb, r.ib, r.ii, idx, tg, c.sp[3], c.sp[4], c.sp[5],
                                         ev); });
      return 0;
    }
    default:
      return RAMP_E_UNSUPPORTED;
  }
}

int generate(Run& r, const RampSource& s, int32_t num_sim, int32_t seed) {
  const float2 md(s.p[0], s.p[1]), td(s.p[2], s.p[3]);
  const float target_dist = s.p[4], E_min = s.p[5], E_max = s.p[6];
  switch (s.kind) {
    case RAMP_SRC_FLAT:
      launch(r.n, [&] { k_flat::generate_neutrons(r.nb, r.ib, md, td, target_dist, E_min, E_max,
                                                  num_sim, seed); });
      return 0;
    case RAMP_SRC_CONT:
      launch(r.n, [&] { k_cont::generate_neutrons(r.nb, r.ib, md, td, target_dist, E_min, E_max,
                                                  s.p[7], s.p[8], s.p[9], s.p[10], s.p[11],
                                                  s.p[12], s.p[13], num_sim, seed); });
      return 0;
    case RAMP_SRC_ISIS: {
      const int nt = (int)s.table_len[1], ne = (int)s.table_len[2];
      /* the scans read the flux table for n_t n_e entries (one energy row
         more than it holds) and both tables one entry before their start
         for a deviate below the first value */
      const int64_t pad = (int64_t)nt + 16;
      Padded flux(s.table[0], s.table_len[0], pad, 2 * pad);
      Padded tb(s.table[1], s.table_len[1], 16, 16);
      Padded eb(s.table[2], s.table_len[2], 16, 16);
      Padded ei(s.table[3], s.table_len[3], 16, 16);
      launch(r.n, [&] { k_isis::generate_neutrons(r.nb, r.ib, md, td, target_dist, E_min, E_max,
                                                  nt, ne, flux.p(), tb.p(), eb.p(), ei.p(),
                                                  s.p[14], s.p[13], 0.0f, num_sim, seed); });
      return 0;
    }
    default:
      return RAMP_E_UNSUPPORTED;
  }
}

}  // namespace

extern "C" {

/* One chunk of Instrument.execute (mcramp.py:442-455) through the
 * reference's own kernels: records [n,16], intersections [n,8], index
 * buffer [n] (host, as oracle_execute_chunk); tallies are host pointers. */
int refcl_execute_chunk(const RampSource* src, const RampComp* comps, int n_comps,
                        const RampBlock* blocks, int n_blocks, float* neutrons, float* isect,
                        uint32_t* iidx, int64_t n, int32_t num_sim, int32_t seed, int threads,
                        uint64_t* oob_out) {
  if (!src || !neutrons || !isect || !iidx || n < 0) return RAMP_E_INVALID;
  if (threads > 0) omp_set_num_threads(threads);
  static_assert(sizeof(float16) == 64 && sizeof(float8) == 32, "record layout");
  Run r;
  r.nb = reinterpret_cast<float16*>(neutrons);
  r.ib = reinterpret_cast<float8*>(isect);
  r.ii = iidx;
  r.n = n;
  int rc = generate(r, *src, num_sim, seed);
  if (rc) return rc;
  for (int b = 0; b < n_blocks; ++b) {
    const RampBlock& B = blocks[b];
    if (B.first < 0 || B.first + B.count > n_comps) return RAMP_E_INVALID;
    if (B.linear) {
      for (int j = B.first; j < B.first + B.count; ++j) {
        transform(r, comps[j]);
        if ((rc = geometry(r, comps[j]))) return rc;
        terminate(r, comps[j]);
        if ((rc = scatter(r, comps[j]))) return rc;
        untransform(r, comps[j]);
      }
    } else {
      for (int e = 0; e < B.multi; ++e) {
        for (int j = B.first; j < B.first + B.count; ++j) {
          transform(r, comps[j]);
          if ((rc = geometry(r, comps[j]))) return rc;
          untransform(r, comps[j]);
        }
        for (int j = B.first; j < B.first + B.count; ++j) {
          transform(r, comps[j]);
          if ((rc = scatter(r, comps[j]))) return rc;
          untransform(r, comps[j]);
        }
      }
    }
  }
  if (oob_out) *oob_out = r.oob;
  return RAMP_OK;
}

}  // extern "C"
