"""CUDA-graph capture of a whole trace.

``Instrument.execute`` (mcramp.py:403-455) issues, for every chunk, one
source draw plus one launch per component (plain path) or one persistent
launch (fused path), and draws each chunk's seed on the host from Python's
``random`` (MFlat/MCont ``randint(0, 4096)``, flat_mod.py:32).  ``capture``
records that sequence once into a CUDA graph whose chunk seeds live in
device memory: before each chunk a one-thread kernel (``ramp_seed_advance``)
draws the next seed in [0, 4096] from a 64-bit LCG, and the trace kernels
read it when they run.  Every ``replay()`` is then one graph launch that
traces N new histories, with no host work per chunk and no Python ``random``
draws; tallies accumulate exactly as repeated ``execute`` calls do.

The chunk seeds of a graph are a deterministic function of its LCG state
(``state``): ``chunk_seeds(k)`` lists the next k seeds on the host, so a
replay can be reproduced eagerly by passing the same seeds.

Descriptor values are read from the plan's device copy on the fused path,
so parameter changes (``ramp_plan_set_param``) reach later replays; the
plain path passes linear components by value at capture time, so changing
a parameter after capturing a plain-path graph needs a new capture (replay
raises).
"""
import ctypes

import torch

from . import _abi

LCG_A = 6364136223846793005
LCG_C = 1442695040888963407
MAX_CHUNKS = 4096


def lcg_seeds(state, k):
    """The next k chunk seeds of an LCG with this 64-bit state, as
    ramp_seed_advance draws them, and the state after them."""
    out = []
    x = int(state) & (2**64 - 1)
    for _ in range(k):
        x = (x * LCG_A + LCG_C) & (2**64 - 1)
        out.append((x >> 33) % 4097)
    return out, x


class TraceGraph:
    """One captured trace of N histories; see ``capture``."""

    def __init__(self, inst, graph, seed_buf, n_chunks, path, epoch, keep):
        self.inst = inst
        self.graph = graph
        self.seed_buf = seed_buf
        self.n_chunks = n_chunks
        self.path = path
        self._epoch = epoch
        self._keep = keep        # buffers the graph's kernels address

    @property
    def state(self):
        """Current 64-bit LCG state (device read; synchronises)."""
        w = self.seed_buf[2:4].cpu().numpy().view("uint64")
        return int(w[0])

    def set_state(self, state):
        x = int(state) & (2**64 - 1)
        lo, hi = x & 0xffffffff, x >> 32
        vals = [0, 0, lo - (1 << 32) if lo >= 1 << 31 else lo,
                hi - (1 << 32) if hi >= 1 << 31 else hi]
        self.seed_buf.copy_(torch.tensor(vals, dtype=torch.int32))

    def chunk_seeds(self, replays=1):
        """Seeds the next ``replays`` replays will use, chunk by chunk."""
        return lcg_seeds(self.state, replays * self.n_chunks)[0]

    def replay(self):
        if self.path == "plain" and getattr(self.inst, "_param_epoch", 0) != self._epoch:
            raise RuntimeError("a parameter changed after this plain-path graph was captured; "
                               "capture it again")
        self.graph.replay()

    def check(self):
        """Synchronise and fold the device status into the instrument
        (cap flags, dropped out-of-range tally writes)."""
        lib = self.inst._lib()
        torch.cuda.synchronize(self.inst.device)
        self.inst._check_status(lib, self.inst.plan())


def capture(inst, N, path="fused", rng="reference", run_seed=0, tune=None, chunk=None,
            state=None):
    """Capture ``inst.execute(N, path=..., rng=..., ...)`` as a CUDA graph.

    state : initial 64-bit LCG state of the chunk seeds (default: drawn from
            Python's ``random``).
    """
    import random

    lib = inst._lib()
    plan = inst.plan()
    N = int(N)
    if N <= 0:
        raise ValueError("N must be positive")
    buf_max = int(chunk) if chunk else inst.chunk_size(None)
    n_chunks = (N + buf_max - 1) // buf_max
    if n_chunks > MAX_CHUNKS:
        raise ValueError("%d chunks: a graph holds at most %d" % (n_chunks, MAX_CHUNKS))
    if path not in ("plain", "fused"):
        raise ValueError("path must be 'plain' or 'fused'")
    tuned = None
    if tune == "auto":
        tune = None
        if path == "fused":
            from . import autotune
            tune = autotune.tune(inst, rng=rng)
    if tune is not None:
        tuned = _abi.tune_struct(tune)
    dev = inst.device
    first = min(N, buf_max)
    with torch.cuda.device(dev):
        seed_buf = torch.zeros(4, dtype=torch.int32, device=dev)
        keep = [seed_buf]
        st = carry = None
        if path == "plain":
            st = inst._alloc_state(first)
            keep += [inst.state, inst.iidx]
        elif N > buf_max:
            carry = torch.zeros((2, first), dtype=torch.float32, device=dev)
            keep.append(carry)
        rngd = _abi.RampRng()
        rngd.mode = {"reference": 0, "native": 1}[rng]
        rngd.run_seed = int(run_seed) & 0xffffffff
        rngd.seed_dev = seed_buf.data_ptr()
        if path == "fused" and tune and any(int(tune.get(k, 0)) > 0
                                            for k in ("split", "walk", "cull")):
            keep.append(inst._survivors(lib, plan, first))   # allocated before the capture
        stream = inst.queue if inst.queue is not None else torch.cuda.Stream(dev)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            sp = ctypes.c_void_p(stream.cuda_stream)
            if path == "plain":
                inst.state.zero_()
                inst.iidx.zero_()
            elif carry is not None:
                carry.zero_()
            remaining = N
            while remaining > 0:
                torun = buf_max if remaining > buf_max else remaining
                remaining -= torun
                _abi.check(lib, lib.ramp_seed_advance(ctypes.c_void_p(seed_buf.data_ptr()), sp),
                           "ramp_seed_advance")
                if path == "plain":
                    rc = lib.ramp_trace_plain(plan, ctypes.byref(st), torun, torun, 0,
                                              ctypes.byref(rngd), sp)
                    _abi.check(lib, rc, "ramp_trace_plain")
                else:
                    sbp = iip = None
                    if carry is not None:
                        sbp = ctypes.c_void_p(carry[0].data_ptr())
                        iip = ctypes.c_void_p(carry[1].data_ptr())
                    rc = lib.ramp_trace_fused(plan, torun, torun, 0, ctypes.byref(rngd), sbp,
                                              iip, ctypes.byref(tuned) if tuned else None, sp)
                    _abi.check(lib, rc, "ramp_trace_fused")
        inst.last_chunk = N - (n_chunks - 1) * buf_max
    tg = TraceGraph(inst, g, seed_buf, n_chunks, path, getattr(inst, "_param_epoch", 0), keep)
    tg.set_state(random.getrandbits(64) if state is None else state)
    return tg
