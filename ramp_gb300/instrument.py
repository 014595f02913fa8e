"""Instrument facade (mcramp/mcramp.py:254-455).

The instrument file is read by ramp_gb300.idf (the reference's IDF grammar
and index rules); this module keeps the reference's chunking (chunk =
max_mem_alloc / 256 neutrons, a random.randint(0, 4096) seed per chunk,
weights 1/N_chunk) and its results API (data, save, plot).  Execution goes through libramp_cuda.so:
``path="plain"`` launches one kernel per component (the reference's call
structure), ``path="fused"`` runs the whole chain in one persistent kernel.
There is no CPU fallback: without a CUDA device or without the library,
execute() raises.
"""
import logging
import warnings

import numpy as np
import torch

from . import _abi, idf
from .idf import frame_rotate  # noqa: F401  (module-level API, mcramp.py:457)
from .shard import chunk_slices
from .scat.sprim import _device

log = logging.getLogger("ramp_gb300")


def build_kernel(filename, ctx=None):
    """mcramp.build_kernel (mcramp.py:13-17) compiles a user OpenCL kernel;
    there is no OpenCL runtime here.  User plugins subclass GPrim/SPrim and
    reuse the built-in kernels through their descriptor slots."""
    raise NotImplementedError("OpenCL kernels are not supported; ramp_gb300 runs built-in "
                              "CUDA kernels selected by the plugin's descriptor kind")


class Instrument:
    """An instrument built from an IDF (mcramp.py:254-455).

    Parameters
    ----------
    fn : str
        Instrument definition file name.
    ctx : torch.device, str, int or None
        Device for tallies and neutron state (the reference takes an OpenCL
        context here).  None selects cuda:0 when available.
    queue : torch.cuda.Stream or None
        Stream the kernels are launched on (None: the current stream).
    **kwargs
        Values for the $...$ variables of the IDF.
    """

    def __init__(self, fn, ctx=None, queue=None, **kwargs):
        self.ctx = ctx
        self.queue = queue
        self.device = _device(ctx)
        self.fn = fn
        self.blocks = idf.load(fn, self, self.device, kwargs)
        self._plan = None
        self._keep = []
        self.state = None
        self.iidx = None
        self.last_chunk = 0
        self.oob_drops = 0
        self.status_flags = 0

    @property
    def source(self):
        for block in self.blocks:
            if block.source is not None:
                return block.source
        raise ValueError("instrument has no source component")

    # ------------------------------------------------------------------
    # descriptors
    # ------------------------------------------------------------------
    def components(self):
        """(name, component dict) for every non-source component in order."""
        out = []
        for block in self.blocks:
            for name, comp in block.components.items():
                out.append((name, comp))
        return out

    def descriptors(self, keep=None):
        """POD descriptors (RampSource, RampComp array, RampBlock array) of
        this instrument; host tables are kept alive in ``keep``."""
        keep = self._keep if keep is None else keep
        src = self.source.descriptor()
        comps = []
        blocks = []
        for block in self.blocks:
            first = len(comps)
            for name, comp in block.components.items():
                c = _abi.RampComp()
                c.idx = comp["idx"]
                c.restore = int(comp["restore_neutron"])
                for k in range(3):
                    c.pos[k] = comp["pos"][k]
                    c.rot[k] = comp["rot"][k]
                comp["geom_kernel"].fill(c, keep)
                comp["scat_kernel"].fill(c, keep)
                if c.geom == 0 or c.scat == 0:
                    raise TypeError("component %s: plugin classes must set a kind" % name)
                comps.append(c)
            b = _abi.RampBlock()
            b.first = first
            b.count = len(comps) - first
            b.linear = 1 if block.linear else 0
            b.multi = int(block.multi)
            blocks.append(b)
        carr = (_abi.RampComp * max(1, len(comps)))(*comps)
        barr = (_abi.RampBlock * max(1, len(blocks)))(*blocks)
        return src, carr, len(comps), barr, len(blocks)

    def tallies(self):
        out = []
        for _, comp in self.components():
            out.extend(comp["scat_kernel"].tallies())
        return out

    def reset_tallies(self):
        """Zero every detector (the reference never resets them)."""
        for t in self.tallies():
            t.zero_()

    # ------------------------------------------------------------------
    # checkpoint / resume (no reference counterpart)
    # ------------------------------------------------------------------
    def checkpoint(self):
        """The state a run resumes from between execute() calls: a host
        copy of every tally and the state of Python's ``random``, from which
        execute() draws each chunk's seed (flat_mod.py:32).  Histories are
        keyed by (chunk seed, index), so a run restored from this state and
        continued gives the tallies the uninterrupted run would."""
        import random
        return {"format": "ramp_gb300 checkpoint 1",
                "tallies": [t.detach().to("cpu").clone() for t in self.tallies()],
                "random": random.getstate()}

    def restore(self, state):
        """Load tallies and the chunk-seed generator from checkpoint().
        The generator is Python's process-wide ``random`` (as the reference
        draws its chunk seeds from it): restoring rewinds it for every
        instrument and every other user of ``random`` in the process."""
        import random
        if state.get("format") != "ramp_gb300 checkpoint 1":
            raise ValueError("not a ramp_gb300 checkpoint")
        mine = self.tallies()
        if len(state["tallies"]) != len(mine) or any(
                a.shape != b.shape for a, b in zip(state["tallies"], mine)):
            raise ValueError("the checkpoint's tallies do not match this instrument")
        for dst, src in zip(mine, state["tallies"]):
            dst.copy_(src)
        random.setstate(state["random"])

    def save_checkpoint(self, path):
        torch.save(self.checkpoint(), path)

    def load_checkpoint(self, path):
        self.restore(torch.load(path))

    # ------------------------------------------------------------------
    # execution
    # ------------------------------------------------------------------
    def _lib(self):
        if self.device.type != "cuda":
            raise RuntimeError("Instrument.execute needs a CUDA device (ctx=%s)" % self.device)
        return _abi.load()

    def plan(self):
        if self._plan is None:
            lib = self._lib()
            with torch.cuda.device(self.device):
                src, carr, nc, barr, nb = self.descriptors()
                h = _abi.ctypes.c_void_p()
                _abi.check(lib, lib.ramp_plan_create(_abi.ctypes.byref(src), carr, nc, barr, nb,
                                                     _abi.ctypes.byref(h)), "ramp_plan_create")
                self._plan = h
                self._lib_handle = lib
        return self._plan

    def __del__(self):
        try:
            if self._plan is not None:
                self._lib_handle.ramp_plan_destroy(self._plan)
                self._plan = None
        except Exception:
            pass

    def max_mem_alloc_size(self):
        """Stand-in for CL_DEVICE_MAX_MEM_ALLOC_SIZE: a quarter of the
        device memory, the value NVIDIA's OpenCL driver reports."""
        return torch.cuda.get_device_properties(self.device).total_memory // 4

    def chunk_size(self, buf_max_mod=None):
        m = self.max_mem_alloc_size()
        return int(m / 8 / 32 / buf_max_mod) if buf_max_mod is not None else int(m / 8 / 32)

    def _stream_ptr(self):
        s = self.queue if self.queue is not None else torch.cuda.current_stream(self.device)
        return _abi.ctypes.c_void_p(s.cuda_stream)

    def _survivors(self, lib, plan, n):
        """The survivor buffer of split fused launches of up to n histories
        (RampTune split, walk, cull): device memory from PyTorch's caching
        allocator, allocated on this instrument's stream and handed to the
        plan (ramp_plan_set_survivors), so that a new Instrument reuses the
        memory of an earlier one instead of allocating gigabytes again."""
        need = int(lib.ramp_survivor_bytes(int(n)))
        buf = getattr(self, "_surv_buf", None)
        if buf is None or buf.numel() < need:
            if self.queue is not None:
                with torch.cuda.stream(self.queue):
                    buf = torch.empty(need, dtype=torch.uint8, device=self.device)
            else:
                buf = torch.empty(need, dtype=torch.uint8, device=self.device)
            _abi.check(lib, lib.ramp_plan_set_survivors(plan, _abi.ctypes.c_void_p(buf.data_ptr()),
                                                        buf.numel()), "ramp_plan_set_survivors")
            self._surv_buf = buf       # the previous buffer, if any, is released after the swap
        return self._surv_buf

    def _alloc_state(self, n):
        stride = (n + 31) // 32 * 32
        self.state = torch.zeros((_abi.NLANES, stride), dtype=torch.float32, device=self.device)
        self.iidx = torch.zeros(stride, dtype=torch.int32, device=self.device)
        st = _abi.RampState()
        st.soa = self.state.data_ptr()
        st.iidx = self.iidx.data_ptr()
        st.stride = stride
        return st

    def execute(self, N, buf_max_mod=None, debug=False, trace=False, path="plain",
                rng="reference", run_seed=0, tune=None, chunk=None, shard=None):
        """Trace N neutron histories (mcramp.py:403-455).

        path : "plain" (one kernel per component) or "fused" (one
               persistent kernel for the whole chain).
        rng  : "reference" reproduces the reference's per-draw Threefry
               stream; "native" uses all four words of each block.
        tune : fused launch configuration: a dict of RampTune fields
               (block, blocks_per_sm, chunk, privatize, split, streams,
               walk, cull) or "auto" for the cached autotuner choice
               (ramp_gb300.autotune).
        chunk: override the chunk size (default max_mem_alloc / 256).
        shard: (rank, world) — trace only this rank's contiguous slice of
               every chunk, keyed by global index and weighted by the full
               chunk size, so the sum of all ranks' tallies equals a
               single-device run (the histogram sum is the caller's
               exchange step, e.g. torch.distributed.all_reduce).
        """
        events = self.event_components()
        hosts = self.host_components()
        if (events or hosts) and path != "plain":
            raise ValueError("SRescal and MCPL components act per neutron index: use path='plain'")
        lib = self._lib()
        plan = self.plan()
        N = int(N)
        buf_max = int(chunk) if chunk else self.chunk_size(buf_max_mod)
        rngd = _abi.RampRng()
        rngd.mode = {"reference": 0, "native": 1}[rng]
        rngd.run_seed = int(run_seed) & 0xffffffff
        tuned = None
        if tune == "auto":
            if path != "fused":
                tune = None
            else:
                from . import autotune
                tune = autotune.tune(self, rng=rng)
        if tune is not None:
            tuned = _abi.tune_struct(tune)
        if trace:
            warnings.warn("trace=True (visualisation lines) is not supported; ignored")
        rank, world = shard if shard is not None else (0, 1)
        slices = chunk_slices(N, buf_max, rank, world)
        first = max(1, max(nloc for _, _, nloc in slices))
        src = self.source
        with torch.cuda.device(self.device):
            stream = self._stream_ptr()
            for j, sc in events:
                buf = sc.prepare(first, self.device)
                _abi.check(lib, lib.ramp_plan_set_buffer(plan, j, _abi.ctypes.c_void_p(buf.data_ptr()),
                                                         buf.numel()), "ramp_plan_set_buffer")
            if path == "plain":
                st = self._alloc_state(first)
            elif path == "fused":
                carry = None
                if tune and any(int(tune.get(k, 0)) > 0 for k in ("split", "walk", "cull")):
                    self._survivors(lib, plan, first)
                if N > buf_max:
                    # per index: final RNG counter (float) and index buffer (uint32)
                    carry = torch.zeros((2, first), dtype=torch.float32, device=self.device)
            else:
                raise ValueError("path must be 'plain' or 'fused'")
            for torun, lo, nloc in slices:
                seed = src.next_seed()          # every rank draws every chunk's seed
                rngd.tid_base = lo
                self.last_chunk = nloc
                if nloc == 0:
                    continue
                if path == "plain":
                    for _, sc in events:
                        sc.begin_chunk()
                    if hosts:
                        self._trace_with_hosts(lib, plan, st, nloc, torun, seed, rngd, stream,
                                               hosts)
                    else:
                        rc = lib.ramp_trace_plain(plan, _abi.ctypes.byref(st), nloc, torun, seed,
                                                  _abi.ctypes.byref(rngd), stream)
                        _abi.check(lib, rc, "ramp_trace_plain")
                    for _, sc in events:
                        sc.reduce(self.state[_abi.LANE["se"]], nloc)
                    if debug:
                        torch.cuda.synchronize(self.device)
                        alive = self.state[:, :nloc][_abi.LANE["die"]] == 0
                        print("Neutron output after chunk (alive records):")
                        print(self.state[:, :nloc][:, alive].T.cpu().numpy())
                else:
                    sbp = iip = None
                    if carry is not None:
                        sbp = _abi.ctypes.c_void_p(carry[0].data_ptr())
                        iip = _abi.ctypes.c_void_p(carry[1].data_ptr())
                    rc = lib.ramp_trace_fused(plan, nloc, torun, seed, _abi.ctypes.byref(rngd),
                                              sbp, iip,
                                              _abi.ctypes.byref(tuned) if tuned else None,
                                              stream)
                    _abi.check(lib, rc, "ramp_trace_fused")
                self.last_chunk = nloc
            self._check_status(lib, plan)

    def capture(self, N, path="fused", rng="reference", run_seed=0, tune=None, chunk=None,
                state=None):
        """``execute(N, ...)`` captured as a CUDA graph whose replays draw
        their chunk seeds on the device (ramp_gb300.graph.capture)."""
        from .graph import capture
        return capture(self, N, path=path, rng=rng, run_seed=run_seed, tune=tune, chunk=chunk,
                       state=state)

    def host_components(self):
        """(descriptor index, plugin) of the components whose scattering runs
        on the host (SMCPLOut, SMCPLIn)."""
        out = []
        j = 0
        for block in self.blocks:
            for name, comp in block.components.items():
                if getattr(comp["scat_kernel"], "kind", None) == _abi.S_HOST:
                    out.append((j, comp["scat_kernel"]))
                j += 1
        return out

    def _trace_with_hosts(self, lib, plan, st, n, num_sim, seed, rngd, stream, hosts):
        """One plain-path chunk with host components: the moderator, then
        every block; a linear block holding host components runs in pieces
        around each host action (mcramp.py:124-157)."""
        ct = _abi.ctypes
        _abi.check(lib, lib.ramp_generate(plan, ct.byref(st), n, num_sim, seed, ct.byref(rngd),
                                          stream), "ramp_generate")
        host_at = dict(hosts)
        first = 0
        for b, block in enumerate(self.blocks):
            count = len(block.components)
            inside = [j for j in range(first, first + count) if j in host_at]
            if not inside:
                _abi.check(lib, lib.ramp_run_block(plan, b, ct.byref(st), n, ct.byref(rngd),
                                                   stream), "ramp_run_block")
            else:
                k = first
                for j in inside:
                    _abi.check(lib, lib.ramp_run_components(plan, k, j, ct.byref(st), n,
                                                            ct.byref(rngd), stream),
                               "ramp_run_components")
                    _abi.check(lib, lib.ramp_component_enter(plan, j, ct.byref(st), n,
                                                             ct.byref(rngd), stream),
                               "ramp_component_enter")
                    host_at[j].host_action(self, st, n)
                    _abi.check(lib, lib.ramp_component_leave(plan, j, ct.byref(st), n, stream),
                               "ramp_component_leave")
                    k = j + 1
                _abi.check(lib, lib.ramp_run_components(plan, k, first + count, ct.byref(st), n,
                                                        ct.byref(rngd), stream),
                           "ramp_run_components")
            first += count

    def event_components(self):
        """(descriptor index, plugin) of the components that record one
        event per neutron index (SRescal)."""
        out = []
        j = 0
        for block in self.blocks:
            for name, comp in block.components.items():
                if getattr(comp["scat_kernel"], "kind", None) == _abi.S_RESCAL:
                    out.append((j, comp["scat_kernel"]))
                j += 1
        return out

    def _check_status(self, lib, plan):
        flags = _abi.ctypes.c_uint32()
        oob = _abi.ctypes.c_uint64()
        _abi.check(lib, lib.ramp_plan_status(plan, _abi.ctypes.byref(flags),
                                             _abi.ctypes.byref(oob)), "ramp_plan_status")
        self.oob_drops += oob.value
        self.status_flags |= flags.value
        if flags.value & (_abi.F_GUIDE_CAP | _abi.F_POWDER_CAP | _abi.F_BVH_STACK):
            warnings.warn("device status flags 0x%x: a bounded loop hit its cap and the "
                          "affected neutrons were terminated" % flags.value)
        if oob.value:
            log.debug("%d tally writes fell outside their buffers and were dropped", oob.value)

    def neutron_state(self):
        """Final records of the last chunk as an array [n, 16] (the
        reference's float16 layout) and the index buffer."""
        if self.state is None:
            raise RuntimeError("no plain-path state (run execute(path='plain') first)")
        n = self.last_chunk
        return (self.state[:, :n].T.contiguous().cpu().numpy(),
                self.iidx[:n].cpu().numpy().view(np.uint32))

    # ------------------------------------------------------------------
    # results
    # ------------------------------------------------------------------
    def data(self):
        """name -> data of every component (mcramp.py:281-293)."""
        return {name: comp["scat_kernel"].data(self.queue) for name, comp in self.components()}

    def plot(self):
        from matplotlib.pyplot import show
        for _, comp in self.components():
            comp["scat_kernel"].plot(self.queue)
        show()

    def save(self):
        for _, comp in self.components():
            comp["scat_kernel"].save(self.queue)

    def visualise(self, *args, **kwargs):
        raise NotImplementedError("instrument visualisation is not part of ramp_gb300")
