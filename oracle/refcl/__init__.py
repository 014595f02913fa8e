"""TEST INFRASTRUCTURE ONLY — the reference's own OpenCL kernels run on the
host (oracle/refcl/driver.cpp through clshim.h; built by
oracle/refcl/build.py from a RAMP checkout, never shipped).

``run(inst, N, math=...)`` traces N histories of an Instrument built with
ctx="cpu" through the reference kernels in the reference's sequencing,
drawing per-chunk seeds from Python's ``random`` as the oracle does, and
returns the last chunk's records.  It is what pins the oracle's
restatement (oracle/oracle.cpp) to the reference's kernel code; only the
tests and the golden-vector generator use it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_libs = {}


def available():
    """The reference's kernels can be built here: from the checkout, or from
    the sources generated from it into oracle/_ref/refcl_src, on a machine
    whose architecture the reference's Random123 accepts."""
    return _build.supported_here() and (
        os.path.isdir(os.path.join(_build.reference_root(), "mcramp")) or
        _build.generated_sources_present())


def unavailable_reason():
    import platform
    if not _build.supported_here():
        return _build.UNSUPPORTED_REASON % platform.machine()
    return "no reference checkout and no sources generated from one"


def checkout_available():
    return os.path.isdir(os.path.join(_build.reference_root(), "mcramp"))


def lib(math="rmath"):
    if math not in _libs:
        paths = _build.build()
        if paths is None:
            return None
        L = ctypes.CDLL(paths[math])
        P = ctypes.c_void_p
        L.refcl_execute_chunk.restype = ctypes.c_int
        L.refcl_execute_chunk.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, P, P, P,
                                          ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int, P]
        _libs[math] = L
    return _libs[math]


class Result:
    def __init__(self, neutrons, isect, iidx, oob):
        self.neutrons = neutrons    # [n, 16] float32, final chunk
        self.isect = isect          # [n, 8]
        self.iidx = iidx            # [n] uint32
        self.oob = oob              # nonzero-weight tally writes past the buffers


def run(inst, N, chunk=None, math="rmath", threads=0, seeds=None):
    """Trace N histories of ``inst`` (ctx="cpu") through the reference
    kernels; tallies accumulate into the instrument's host tallies."""
    L = lib(math)
    if L is None:
        raise RuntimeError("the reference checkout is not available")
    for t in inst.tallies():
        if t.device.type != "cpu":
            raise ValueError("needs an Instrument with ctx='cpu'")
    if inst.host_components():
        raise NotImplementedError("no host components (MCPL in/out) here")
    N = int(N)
    buf_max = int(chunk) if chunk else N
    first = min(N, buf_max)
    events = inst.event_components()
    import torch
    for _, sc in events:
        sc.prepare(first, torch.device("cpu"))
    keep = []
    src, carr, nc, barr, nb = inst.descriptors(keep)
    neutrons = np.zeros((first, 16), dtype=np.float32)
    isect = np.zeros((first, 8), dtype=np.float32)
    iidx = np.zeros(first, dtype=np.uint32)
    oob = ctypes.c_uint64()
    tot = 0
    remaining, k, last = N, 0, 0
    while remaining > 0:
        torun = buf_max if remaining > buf_max else remaining
        remaining -= torun
        seed = inst.source.next_seed() if seeds is None else int(seeds[k])
        k += 1
        for _, sc in events:
            sc.begin_chunk()
        rc = L.refcl_execute_chunk(ctypes.addressof(src), ctypes.addressof(carr), nc,
                                   ctypes.addressof(barr), nb, neutrons.ctypes.data,
                                   isect.ctypes.data, iidx.ctypes.data, torun, torun, seed,
                                   int(threads), ctypes.addressof(oob))
        if rc != 0:
            raise RuntimeError("refcl_execute_chunk failed (%d)" % rc)
        tot += oob.value
        last = torun
        if events:
            se = torch.from_numpy(neutrons[:, 14].copy())
            for _, sc in events:
                sc.reduce(se, torun)
    return Result(neutrons[:last], isect[:last], iidx[:last], tot)
