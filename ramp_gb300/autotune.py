"""Launch-configuration autotuner for the fused path.

The fused kernel's result does not depend on its launch configuration (the
RNG is counter-based and keyed by neutron index), so the configuration can
be chosen purely for speed.  ``tune(inst)`` times short fused runs of the
instrument over the candidates (register cap = minimum CTAs per SM, and
the span of neutrons a task covers) and keeps the fastest; results are
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

CANDIDATES = [dict(blocks_per_sm=b, chunk=c) for b in (2, 3, 4) for c in (0, 4096, 16384)]


def cache_path():
    return os.environ.get("RAMP_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "ramp_gb300", "autotune.json")


def signature(inst, rng):
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
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _time_config(lib, plan, n, rng, cfg, stream, reps=2):
    tune = _abi.RampTune(0, int(cfg.get("blocks_per_sm", 0)), int(cfg.get("chunk", 0)), 0)
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


def tune(inst, n_probe=2_000_000, rng="reference", candidates=None, force=False):
    """Best fused launch configuration for ``inst`` (a dict for
    Instrument.execute(tune=...)); measured once per GPU and instrument
    structure, then read from the cache."""
    key = signature(inst, rng)
    cache = _load()
    if not force and key in cache:
        return dict(cache[key]["config"])
    lib = inst._lib()
    plan = inst.plan()
    saved = [t.clone() for t in inst.tallies()]
    rngd = _abi.RampRng({"reference": 0, "native": 1}[rng], 0, 0, 0)
    results = []
    with torch.cuda.device(inst.device):
        stream = torch.cuda.current_stream(inst.device)
        for cfg in (candidates or CANDIDATES):
            results.append((_time_config(lib, plan, n_probe, rngd, cfg, stream), cfg))
        torch.cuda.synchronize(inst.device)
        for t, s in zip(inst.tallies(), saved):
            t.copy_(s)
        inst._check_status(lib, plan)
    results.sort(key=lambda x: x[0])
    best = results[0][1]
    cache[key] = {"config": best, "ms": results[0][0], "n_probe": n_probe,
                  "all": [[ms, c] for ms, c in results]}
    _save(cache)
    return dict(best)
