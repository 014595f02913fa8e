"""TEST INFRASTRUCTURE ONLY — the CPU oracle.

A ctypes wrapper around oracle/oracle.cpp, the CPU restatement of RAMP's
OpenCL kernels (reference sequencing: five passes per linear component over
array-of-structs records, reference RNG keying).  Only tests/, the smoke
check of __graft_entry__ and the cpu_baseline leg of bench.py use it; the
product path (ramp_gb300) never imports it.

``run(inst, N, ...)`` reproduces Instrument.execute's chunk loop
(mcramp.py:403-455) on the CPU for an Instrument whose tallies live in host
memory (ctx="cpu"), drawing the same per-chunk seeds from Python's
``random`` module.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_pins = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.oracle_execute_chunk.restype = ctypes.c_int
        L.oracle_execute_chunk.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, P, P, P,
                                           ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, P,
                                           ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, P, P]
        L.oracle_threefry.argtypes = [P, P, P, ctypes.c_int64]
        L.oracle_rand.restype = ctypes.c_float
        L.oracle_rand.argtypes = [P, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32,
                                  ctypes.c_uint32]
        L.oracle_reflectivity.restype = ctypes.c_float
        L.oracle_reflectivity.argtypes = [ctypes.c_float] * 6
        L.oracle_math.argtypes = [ctypes.c_int, P, P, P, ctypes.c_int64]
        _lib = L
    return _lib


def pins():
    """The reference's own rand.h / ref.h compiled on the host, or None when
    the reference checkout is not available (e.g. on the GPU machine)."""
    global _pins
    if _pins is None:
        path = _build.build_ref_pins()
        if path is None or not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ref_pin_rand.restype = ctypes.c_float
        L.ref_pin_rand.argtypes = [P, ctypes.c_uint]
        L.ref_pin_reflectivity.restype = ctypes.c_float
        L.ref_pin_reflectivity.argtypes = [ctypes.c_float] * 6
        L.ref_pin_threefry.argtypes = [P, P, P, ctypes.c_long]
        _pins = L
    return _pins


def threefry(ctr0, tid):
    ctr0 = np.ascontiguousarray(ctr0, dtype=np.uint32)
    tid = np.ascontiguousarray(tid, dtype=np.uint32)
    out = np.empty_like(ctr0)
    lib().oracle_threefry(ctr0.ctypes.data, tid.ctypes.data, out.ctypes.data, ctr0.size)
    return out


def math(fn, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    bb = None if b is None else np.ascontiguousarray(b, dtype=np.float32)
    out = np.empty_like(a)
    lib().oracle_math(int(fn), a.ctypes.data, None if bb is None else bb.ctypes.data,
                      out.ctypes.data, a.size)
    return out


class Result:
    def __init__(self, neutrons, isect, iidx, flags, oob):
        self.neutrons = neutrons    # [n, 16] float32, final chunk
        self.isect = isect          # [n, 8] float32
        self.iidx = iidx            # [n] uint32
        self.flags = flags
        self.oob = oob


def run(inst, N, chunk=None, rng_mode=0, run_seed=0, variant=0, threads=0, seeds=None,
        tid_base=0, num_sim=None, shard=None):
    """Trace N histories of ``inst`` (an Instrument built with ctx="cpu")
    through the CPU restatement; tallies accumulate into the instrument's
    host tallies.  Returns the final chunk's records.  ``tid_base`` and
    ``num_sim`` describe a shard: records [0, N) are neutrons
    [tid_base, tid_base+N) of a chunk of ``num_sim`` histories.
    ``shard=(rank, world)`` traces rank's part of every chunk of an
    N-history run: the slice [lo, hi) of the first chunk's index range,
    clipped to each chunk's size (the same global indices every chunk,
    so carried RNG counters stay with their index)."""
    import torch  # noqa: F401  (tallies are torch CPU tensors)
    for t in inst.tallies():
        if t.device.type != "cpu":
            raise ValueError("the oracle needs an Instrument with ctx='cpu'")
    N = int(N)
    buf_max = int(chunk) if chunk else N
    first = min(N, buf_max)
    s_lo, s_hi = 0, first
    if shard is not None:
        rank, world = shard
        s_lo, s_hi = first * rank // world, first * (rank + 1) // world
        first = max(1, s_hi - s_lo)
    if inst.host_components():
        raise NotImplementedError("the oracle has no host components (MCPL in/out)")
    events = inst.event_components()
    for _, sc in events:             # per-index event buffers (SRescal)
        sc.prepare(first, torch.device("cpu"))
    keep = []
    src, carr, nc, barr, nb = inst.descriptors(keep)
    neutrons = np.zeros((first, 16), dtype=np.float32)
    isect = np.zeros((first, 8), dtype=np.float32)
    iidx = np.zeros(first, dtype=np.uint32)

    from ramp_gb300._abi import RampRng
    rng = RampRng(int(rng_mode), int(run_seed) & 0xffffffff, int(tid_base), 0)
    flags = ctypes.c_uint32()
    oob = ctypes.c_uint64()
    tot_flags, tot_oob = 0, 0
    remaining = N
    k = 0
    while remaining > 0:
        torun = buf_max if remaining > buf_max else remaining
        remaining -= torun
        seed = inst.source.next_seed() if seeds is None else int(seeds[k])
        k += 1
        nrec, nsim = torun, int(num_sim) if num_sim else torun
        if shard is not None:
            nrec, nsim = max(0, min(s_hi, torun) - s_lo), torun
            rng.tid_base = s_lo
            if nrec == 0:
                last = 0
                continue
        for _, sc in events:
            sc.begin_chunk()
        rc = lib().oracle_execute_chunk(ctypes.addressof(src), ctypes.addressof(carr), nc,
                                        ctypes.addressof(barr), nb, neutrons.ctypes.data,
                                        isect.ctypes.data, iidx.ctypes.data, nrec,
                                        nsim, seed,
                                        ctypes.addressof(rng), int(variant), 0, int(threads),
                                        ctypes.addressof(flags), ctypes.addressof(oob))
        if rc != 0:
            raise RuntimeError("oracle_execute_chunk failed (%d)" % rc)
        tot_flags |= flags.value
        tot_oob += oob.value
        last = nrec
        if events:
            import torch as _t
            se = _t.from_numpy(neutrons[:, 14].copy())
            for _, sc in events:
                sc.reduce(se, nrec)
    return Result(neutrons[:last], isect[:last], iidx[:last], tot_flags, tot_oob)
