"""Launch-configuration autotuner for the fused path.

The fused kernel's result does not depend on its launch configuration (the
RNG is counter-based and keyed by neutron index), so the configuration can
be chosen purely for speed.  ``tune(inst)`` times short fused runs of the
instrument over the candidates (register cap = minimum CTAs per SM, the
span of neutrons a task covers, whether survivors are compacted into
full warps before the first component that less than half of the
histories reach — found by a plain-path pilot, ``survival`` — 128- against
256-thread CTAs, shared-memory private
tallies for chains whose detectors fit, for chains with a mesh the
per-lane mesh walk, and for chains with a run of on-axis disk choppers the
chopper look-ahead, which retires before the run the neutrons that cannot
pass it) and keeps the fastest; results are
cached in a JSON file keyed by GPU name, the instrument's component
structure and the keying mode.  Tuning uses fixed seeds and restores the
instrument's tallies afterwards: it leaves no trace in the results or in
Python's ``random`` state.

Cache location: $RAMP_AUTOTUNE_CACHE, else ~/.cache/ramp_gb300/autotune.json.
"""
import ctypes
import hashlib
import json
import os

import torch

from . import _abi

# the default register cap (4 CTAs per SM) first: near-ties keep the earlier candidate
CANDIDATES = [dict(blocks_per_sm=b, chunk=c) for b in (4, 3) for c in (0, 4096)]
TIE = 0.01        # candidates within 1 % of the fastest count as tied


def cache_path():
    return os.environ.get("RAMP_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "ramp_gb300", "autotune.json")


_MEMO = {}   # signature -> configuration, for the lookups after the first in a process


def signature(inst, rng):
    memo = getattr(inst, "_tune_sig", None)
    if memo is None:
        memo = inst._tune_sig = {}
    if rng in memo:                  # the component structure of an instrument is fixed
        return memo[rng]
    memo[rng] = _signature(inst, rng)
    return memo[rng]


def _signature(inst, rng):
    src, carr, nc, barr, nb = inst.descriptors([])
    kinds = [(carr[j].geom, carr[j].scat) for j in range(nc)]
    blocks = [(barr[k].first, barr[k].count, barr[k].linear, barr[k].multi) for k in range(nb)]
    name = torch.cuda.get_device_name(inst.device)
    h = hashlib.sha1(json.dumps([name, src.kind, kinds, blocks, rng]).encode()).hexdigest()
    return h[:16]


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(cache):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = "%s.%d.tmp" % (p, os.getpid())   # ranks of one job may save at once
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def survival(inst, n=1_000_000, rng="reference", seed=17):
    """Histories alive at the entry of each component, out of n traced on
    the plain path with the chain re-planned as one block per linear
    component (ramp_generate, then ramp_run_block block by block, counting
    live records in between).  Entry i belongs to component i; components
    inside a non-linear block after its first get None.  Adds the pilot's
    histories to the instrument's tallies (callers restore them)."""
    ct = ctypes
    lib = inst._lib()
    keep = []
    src, carr, nc, barr, nb = inst.descriptors(keep)
    blocks, first_of = [], []
    for k in range(nb):
        b = barr[k]
        if b.linear:
            for j in range(b.first, b.first + b.count):
                blocks.append(_abi.RampBlock(j, 1, 1, b.multi))
                first_of.append(j)
        else:
            blocks.append(_abi.RampBlock(b.first, b.count, 0, b.multi))
            first_of.append(b.first)
    barr2 = (_abi.RampBlock * max(1, len(blocks)))(*blocks)
    plan = ct.c_void_p()
    _abi.check(lib, lib.ramp_plan_create(ct.byref(src), carr, nc, barr2, len(blocks),
                                         ct.byref(plan)), "ramp_plan_create")
    alive = [None] * nc
    try:
        dev = inst.device
        stride = (n + 31) // 32 * 32
        soa = torch.zeros((_abi.NLANES, stride), dtype=torch.float32, device=dev)
        iidx = torch.zeros(stride, dtype=torch.int32, device=dev)
        st = _abi.RampState()
        st.soa, st.iidx, st.stride = soa.data_ptr(), iidx.data_ptr(), stride
        rngd = _abi.RampRng({"reference": 0, "native": 1}[rng], 0, 0, 0)
        with torch.cuda.device(dev):
            stream = ct.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            _abi.check(lib, lib.ramp_generate(plan, ct.byref(st), n, n, seed, ct.byref(rngd),
                                              stream), "ramp_generate")
            die = soa[_abi.LANE["die"], :n]
            for b in range(len(blocks)):
                alive[first_of[b]] = int((die == 0).sum())
                _abi.check(lib, lib.ramp_run_block(plan, b, ct.byref(st), n, ct.byref(rngd),
                                                   stream), "ramp_run_block")
            torch.cuda.synchronize(dev)
            flags, oob = ct.c_uint32(), ct.c_uint64()
            lib.ramp_plan_status(plan, ct.byref(flags), ct.byref(oob))
    finally:
        lib.ramp_plan_destroy(plan)
    return alive


def split_point(inst, alive, threshold=0.5):
    """First component at whose entry fewer than ``threshold`` of the
    histories are alive (a valid compaction point), or 0."""
    _, _, nc, barr, nb = inst.descriptors([])
    inside = set()
    for k in range(nb):
        if not barr[k].linear:
            inside.update(range(barr[k].first + 1, barr[k].first + barr[k].count))
    n0 = alive[0] if alive and alive[0] else 0
    for k in range(1, nc):
        if k in inside or alive[k] is None:
            continue
        if n0 and alive[k] < threshold * n0:
            return k
    return 0


def chopper_run_start(inst):
    """First component at which a run of on-axis straight guides and disk
    choppers starts, for the chopper look-ahead (RampTune.cull;
    ramp_chopper_run), or None."""
    keep = []
    _, carr, nc, barr, nb = inst.descriptors(keep)
    lib = _abi.load()
    for k in range(nc):
        if lib.ramp_chopper_run(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, k) > 0:
            return k
    return None


def speed_kept_fraction(inst, n_grid=1 << 20):
    """Fraction of the histories the speed look-ahead of a split launch at
    component 0 keeps (the lean stage A regenerates those): the energies of
    a flat or MCont moderator come from one uniform Threefry word each, so
    this is the share of an even grid of words whose energies
    ramp_debug_speed_cull does not rule out.  1.0 with another source or
    without a run at component 0."""
    import numpy as np
    keep = []
    src, carr, nc, barr, nb = inst.descriptors(keep)
    lib = _abi.load()
    if src.kind not in (_abi.SRC_FLAT, _abi.SRC_CONT) or nc == 0 or \
            lib.ramp_chopper_run(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, 0) <= 0:
        return 1.0
    words = np.ascontiguousarray((np.arange(n_grid, dtype=np.uint64) * (1 << 31) // n_grid
                                  + (1 << 30) // n_grid).astype(np.uint32))
    p = np.ascontiguousarray(np.array(src.p[0:7], dtype=np.float32))
    out = np.zeros(n_grid, np.uint8)
    _abi.check(lib, lib.ramp_debug_speed_cull(ctypes.addressof(carr), nc, ctypes.addressof(barr),
                                              nb, 0, p.ctypes.data, words.ctypes.data, n_grid,
                                              out.ctypes.data, None), "ramp_debug_speed_cull")
    return float(1.0 - out.mean())


def privatizable(inst):
    """Whether a detector of the chain has histograms small enough for the
    shared-memory private tallies of a whole-chain launch (two float
    histograms within 48 KB)."""
    _, carr, nc, _, _ = inst.descriptors([])
    return any(carr[j].scat in (_abi.S_DET1D, _abi.S_DET2D) and
               0 < 2 * carr[j].tally_len <= 12288 for j in range(nc))


def has_mesh(inst):
    """Whether a linear block of the chain holds a GMesh component (the
    candidates then include the per-lane mesh walk, RampTune.walk)."""
    _, carr, nc, barr, nb = inst.descriptors([])
    return any(barr[k].linear and carr[j].geom == _abi.G_MESH
               for k in range(nb) for j in range(barr[k].first, barr[k].first + barr[k].count))


def _time_config(lib, plan, n, rng, cfg, stream, reps=2):
    tune = _abi.tune_struct(cfg)
    best = None
    for r in range(reps + 1):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        rc = lib.ramp_trace_fused(plan, n, n, 17 + r, ctypes.byref(rng), None, None,
                                  ctypes.byref(tune), ctypes.c_void_p(stream.cuda_stream))
        e.record(stream)
        e.synchronize()
        _abi.check(lib, rc, "ramp_trace_fused")
        if r > 0:
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
    return best


def tune(inst, n_probe=40_000_000, rng="reference", candidates=None, force=False):
    """Best fused launch configuration for ``inst`` (a dict for
    Instrument.execute(tune=...)); measured once per GPU and instrument
    structure, then read from the cache."""
    key = signature(inst, rng)
    if not force and key in _MEMO:
        return dict(_MEMO[key])
    cache = _load()
    if not force and key in cache:
        _MEMO[key] = dict(cache[key]["config"])
        return dict(cache[key]["config"])
    lib = inst._lib()
    plan = inst.plan()
    saved = [t.clone() for t in inst.tallies()]
    rngd = _abi.RampRng({"reference": 0, "native": 1}[rng], 0, 0, 0)
    results = []
    split = 0
    if candidates is None:
        split = split_point(inst, survival(inst, min(n_probe, 1_000_000), rng))
        candidates = [dict(c, split=k) for c in CANDIDATES for k in ((0, split) if split else (0,))]
        # 128-thread CTAs at the same threads per SM, with the best split
        candidates += [dict(block=128, blocks_per_sm=2 * b, split=split)
                       for b in (3, 4)]
        if privatizable(inst):
            candidates += [dict(c, privatize=1) for c in CANDIDATES]
        if has_mesh(inst):
            candidates += [dict(c, walk=1) for c in CANDIDATES]
        k0 = chopper_run_start(inst)
        if k0 is not None:
            candidates += [dict(c, split=k0, cull=1) for c in CANDIDATES]
            # 8 before 6 CTAs per SM: probes tie within TIE, 8 measured 3 % faster at 1e8
            candidates += [dict(block=128, blocks_per_sm=2 * b, split=k0, cull=1) for b in (4, 3)]
    with torch.cuda.device(inst.device):
        stream = torch.cuda.current_stream(inst.device)
        for cfg in candidates:
            results.append((_time_config(lib, plan, n_probe, rngd, cfg, stream), cfg))
        torch.cuda.synchronize(inst.device)
        for t, s in zip(inst.tallies(), saved):
            t.copy_(s)
        inst._check_status(lib, plan)
    fastest = min(ms for ms, _ in results)
    # the first candidate (in the order above) within TIE of the fastest:
    # short probes cannot tell near-ties apart
    best_ms, best = next((ms, c) for ms, c in results if ms <= fastest * (1.0 + TIE))
    results.sort(key=lambda x: x[0])
    cache[key] = {"config": best, "ms": best_ms, "n_probe": n_probe, "split_candidate": split,
                  "all": [[ms, c] for ms, c in results]}
    _save(cache)
    _MEMO[key] = dict(best)
    return dict(best)
