"""Batched fused tracing: many variants of one instrument in one launch.

No reference counterpart: RAMP runs one Instrument per execute().  Here a
BatchedInstrument holds one Instrument per variant (same IDF, different
$...$ values, hence different parameters and its own tallies) and traces
all of them, each with its own neutron count, chunk weight 1/N_v and seed,
in one persistent kernel (ramp_trace_batched).  Variant v with keying
"reference" reproduces exactly what Instrument.execute(N_v) would give for
that variant alone with the same seed; "native" adds the variant id to the
Threefry key and uses all four words of each block.
"""
import ctypes

import torch

from . import _abi
from .instrument import Instrument


class BatchedInstrument:
    def __init__(self, fn, variants, ctx=None, queue=None):
        if not variants:
            raise ValueError("BatchedInstrument needs at least one variant")
        self.instruments = [Instrument(fn, ctx, queue, **kw) for kw in variants]
        base = self.instruments[0]
        self.device = base.device
        self.queue = queue
        # the variants' descriptors, built once here (a variant's parameters
        # are fixed at construction, as an Instrument's plan is) and kept,
        # with the host tables they point to, for every execute
        self._keep = []
        self._variants = (_abi.RampVariant * len(self.instruments))()
        kinds = None
        for k, inst in enumerate(self.instruments):
            src, carr, nc, barr, nb = inst.descriptors(self._keep)
            self._keep.append(carr)
            kk = ([(carr[j].geom, carr[j].scat) for j in range(nc)],
                  [(barr[b].first, barr[b].count, barr[b].linear, barr[b].multi)
                   for b in range(nb)])
            if kinds is None:
                kinds = kk
            elif kk != kinds:
                raise ValueError("variant %d has a different component structure" % k)
            self._variants[k].comps = ctypes.cast(carr, ctypes.POINTER(_abi.RampComp))
            self._variants[k].source = src

    def execute(self, counts, rng="native", run_seed=0, seeds=None, tune=None):
        """Trace counts[v] histories of variant v, all in one launch."""
        if len(counts) != len(self.instruments):
            raise ValueError("one count per variant")
        base = self.instruments[0]
        lib = base._lib()
        plan = base.plan()
        nv = len(self.instruments)
        variants = self._variants
        chunk = base.chunk_size()
        for v, inst in enumerate(self.instruments):
            n = int(counts[v])
            if n > chunk:
                raise ValueError("variant %d: %d histories exceed one chunk (%d)" % (v, n, chunk))
            variants[v].n = n
            variants[v].num_sim = max(n, 1)
            variants[v].seed = int(seeds[v]) if seeds is not None else inst.source.next_seed()
        rngd = _abi.RampRng()
        rngd.mode = {"reference": 0, "native": 1}[rng]
        rngd.run_seed = int(run_seed) & 0xffffffff
        tuned = None
        if tune is not None:
            tuned = _abi.tune_struct(tune)
        with torch.cuda.device(self.device):
            stream = base._stream_ptr()
            rc = lib.ramp_trace_batched(plan, variants, nv, ctypes.byref(rngd),
                                        ctypes.byref(tuned) if tuned else None, stream)
            _abi.check(lib, rc, "ramp_trace_batched")
            base._check_status(lib, plan)
        self.variant_seeds = [int(variants[v].seed) for v in range(nv)]

    def data(self):
        return [inst.data() for inst in self.instruments]

    def tallies(self):
        return [inst.tallies() for inst in self.instruments]
