"""ctypes mirror of ``include/ramp.h`` and the loader for ``libramp_cuda.so``.

The structures here are the plain-old-data descriptors the plugin classes
fill (one ``RampComp`` per component, one ``RampSource`` per moderator, one
``RampBlock`` per execution block).  The same descriptors drive the CUDA
library and the CPU oracle used by the tests.
"""
import ctypes
import os

import numpy as np

NLANES = 16
LANE = dict(x=0, y=1, z=2, vx=3, vy=4, vz=5, px=6, py=7, pz=8, p=9, tof=10,
            mc=11, prevcomp=12, sd=13, se=14, die=15)

# kinds (RampSourceKind / RampGeomKind / RampScatKind)
SRC_FLAT, SRC_CONT, SRC_ISIS = 1, 2, 3
G_PLANE, G_CYL_EXT, G_BANANA, G_SPHERE, G_SPHERE_INT, G_BOX, G_ARM, G_MESH = range(1, 9)
(S_ARM, S_GUIDE, S_CHOPPER, S_ISOTROPIC, S_POWDERN, S_DET1D, S_DET2D, S_COUNTER,
 S_BEAMSTOP, S_ATTENUATE, S_MONO, S_POWDER1, S_RESCAL, S_HOST) = range(1, 15)

NGP, NSP, NGI, NSI, NTAB = 12, 24, 4, 12, 12

RAMP_OK = 0
E_INVALID, E_CUDA, E_NOMEM, E_DEVICE, E_UNSUPPORTED, E_RANGE = -1, -2, -3, -4, -5, -6
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory",
          -4: "device status flag raised", -5: "unsupported component",
          -6: "size beyond documented maximum"}

F_GUIDE_CAP, F_POWDER_CAP, F_TALLY_OOB, F_BVH_STACK, F_WORKQ = 1, 2, 4, 8, 16


class RampSource(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("p", ctypes.c_float * 16),
                ("table", ctypes.POINTER(ctypes.c_float) * 4),
                ("table_len", ctypes.c_int64 * 4)]


class RampComp(ctypes.Structure):
    _fields_ = [("geom", ctypes.c_int32), ("scat", ctypes.c_int32),
                ("idx", ctypes.c_uint32), ("restore", ctypes.c_uint32),
                ("pos", ctypes.c_float * 3), ("rot", ctypes.c_float * 3),
                ("gp", ctypes.c_float * NGP), ("sp", ctypes.c_float * NSP),
                ("gi", ctypes.c_int32 * NGI), ("si", ctypes.c_int32 * NSI),
                ("table", ctypes.c_void_p * NTAB), ("table_len", ctypes.c_int64 * NTAB),
                ("tally", ctypes.c_void_p), ("tally_err", ctypes.c_void_p),
                ("tally_len", ctypes.c_int64)]


class RampBlock(ctypes.Structure):
    _fields_ = [("first", ctypes.c_int32), ("count", ctypes.c_int32),
                ("linear", ctypes.c_int32), ("multi", ctypes.c_int32)]


class RampState(ctypes.Structure):
    _fields_ = [("soa", ctypes.c_void_p), ("iidx", ctypes.c_void_p),
                ("stride", ctypes.c_int64)]


class RampRng(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("run_seed", ctypes.c_uint32),
                ("tid_base", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("seed_dev", ctypes.c_void_p)]


class RampVariant(ctypes.Structure):
    _fields_ = [("comps", ctypes.POINTER(RampComp)), ("source", RampSource),
                ("n", ctypes.c_int64), ("num_sim", ctypes.c_int32),
                ("seed", ctypes.c_int32)]


class RampDiffParam(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("comp", ctypes.c_int32)]


DP_GUIDE_R0, DP_GUIDE_QC, DP_GUIDE_ALPHA, DP_GUIDE_M, DP_GUIDE_W, DP_SOURCE_T, \
    DP_POWDER_SIGMA_ABS = range(1, 8)


class RampTune(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("chunk", ctypes.c_int32), ("privatize", ctypes.c_int32),
                ("split", ctypes.c_int32), ("streams", ctypes.c_int32),
                ("walk", ctypes.c_int32), ("cull", ctypes.c_int32)]


TUNE_KEYS = ("block", "blocks_per_sm", "chunk", "privatize", "split", "streams", "walk", "cull")


def tune_struct(tune):
    """RampTune from a dict of launch settings (missing keys: 0 = default)."""
    unknown = set(tune) - set(TUNE_KEYS)
    if unknown:
        raise ValueError("unknown launch settings: %s" % sorted(unknown))
    return RampTune(*[int(tune.get(k, 0)) for k in TUNE_KEYS])


def set_table(comp, slot, arr, keep):
    """Point table slot ``slot`` of ``comp`` at the float32 array ``arr``
    (host memory, kept alive by appending it to ``keep``)."""
    a = np.ascontiguousarray(arr, dtype=np.float32).ravel()
    keep.append(a)
    comp.table[slot] = a.ctypes.data if a.size else None
    comp.table_len[slot] = a.size


# --------------------------------------------------------------------------
# library loading
# --------------------------------------------------------------------------
_HERE = os.path.dirname(os.path.abspath(__file__))
# RAMP_CUDA_LIB selects another build of the library (e.g. an experimental one)
LIB_PATH = os.environ.get("RAMP_CUDA_LIB") or os.path.join(_HERE, "_build", "libramp_cuda.so")
_lib = None

_SIGS = {
    "ramp_version": ([], ctypes.c_int),
    "ramp_last_error": ([ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "ramp_plan_create": ([ctypes.POINTER(RampSource), ctypes.POINTER(RampComp), ctypes.c_int,
                          ctypes.POINTER(RampBlock), ctypes.c_int,
                          ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "ramp_plan_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "ramp_plan_status": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32),
                          ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "ramp_generate": ([ctypes.c_void_p, ctypes.POINTER(RampState), ctypes.c_int64,
                       ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(RampRng),
                       ctypes.c_void_p], ctypes.c_int),
    "ramp_run_block": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(RampState),
                        ctypes.c_int64, ctypes.POINTER(RampRng), ctypes.c_void_p], ctypes.c_int),
    "ramp_trace_plain": ([ctypes.c_void_p, ctypes.POINTER(RampState), ctypes.c_int64,
                          ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(RampRng),
                          ctypes.c_void_p], ctypes.c_int),
    "ramp_trace_fused": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                          ctypes.POINTER(RampRng), ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.POINTER(RampTune), ctypes.c_void_p], ctypes.c_int),
    "ramp_trace_batched": ([ctypes.c_void_p, ctypes.POINTER(RampVariant), ctypes.c_int,
                            ctypes.POINTER(RampRng), ctypes.POINTER(RampTune),
                            ctypes.c_void_p], ctypes.c_int),
    "ramp_trace_batched_noalloc": ([ctypes.c_void_p, ctypes.POINTER(RampVariant), ctypes.c_int,
                                    ctypes.POINTER(RampRng), ctypes.POINTER(RampTune),
                                    ctypes.c_void_p], ctypes.c_int),
    "ramp_plan_set_param": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_float],
                            ctypes.c_int),
    "ramp_adjoint": ([ctypes.c_void_p, ctypes.POINTER(RampDiffParam), ctypes.c_int, ctypes.c_int,
                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                      ctypes.POINTER(RampRng), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
                     ctypes.c_int),
    "ramp_seed_advance": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ramp_plan_reserve": ([ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "ramp_forward_record": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                             ctypes.c_int32, ctypes.POINTER(RampRng), ctypes.c_void_p],
                            ctypes.c_int),
    "ramp_plan_set_buffer": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64],
                             ctypes.c_int),
    "ramp_run_components": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                             ctypes.POINTER(RampState), ctypes.c_int64, ctypes.POINTER(RampRng),
                             ctypes.c_void_p], ctypes.c_int),
    "ramp_component_enter": ([ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(RampState),
                              ctypes.c_int64, ctypes.POINTER(RampRng), ctypes.c_void_p],
                             ctypes.c_int),
    "ramp_component_leave": ([ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(RampState),
                              ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "ramp_gather_alive": ([ctypes.POINTER(RampState), ctypes.c_int64, ctypes.c_uint32,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                           ctypes.c_void_p], ctypes.c_int),
    "ramp_debug_threefry": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "ramp_debug_math": ([ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                         ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "ramp_debug_rng_peak": ([ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p],
                            ctypes.c_int),
    "ramp_debug_l2_peak": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                            ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ramp_debug_atomic_peak": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                ctypes.c_void_p], ctypes.c_int),
    "ramp_bvh_walk_counts": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                              ctypes.c_void_p], ctypes.c_int),
    "ramp_survivor_bytes": ([ctypes.c_int64], ctypes.c_int64),
    "ramp_plan_set_survivors": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "ramp_chopper_run": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                          ctypes.c_int], ctypes.c_int),
    "ramp_debug_speed_cull": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                               ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                               ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ramp_debug_chopper_cull": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
                                ctypes.c_int),
}


def exported_symbols():
    """Names declared in include/ramp.h that the library must export."""
    return list(_SIGS)


def load(path=None):
    """Load libramp_cuda.so (built by ``ramp_gb300.build``).  Raises if it is
    missing: there is no fallback implementation."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libramp_cuda.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
            "g.build()\"` or `python -m ramp_gb300.build`" % p)
    lib = ctypes.CDLL(p)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def last_error(lib):
    buf = ctypes.create_string_buffer(512)
    lib.ramp_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(lib, rc, what):
    if rc != RAMP_OK:
        raise RuntimeError("%s failed (%d, %s): %s" % (what, rc, ERRORS.get(rc, "?"),
                                                         last_error(lib)))
