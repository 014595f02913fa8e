#!/usr/bin/env python
"""Benchmark: neutron histories/s of the LET-like chopper-spectrometer chain
(1e8 histories per step, FP32, reference RNG keying) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 2|3|4|5] [--no-extra]

A step is one Instrument.execute(1e8) of the LET-like instrument (Maxwellian
moderator, 4 supermirror guides, 5 disk choppers, 40-line powder sample,
720 x 1000 banana detector) on the fused path (whole chain in one
persistent kernel).  The plain path (one kernel per component, neutron
state in HBM) is timed beside it on the same histories.  The instrument is
a seeded synthetic stand-in for the reference's LET example.

value: histories/s over all ranks, device-timed (CUDA events per step, L2
flushed between steps by writing a 256 MiB buffer outside the events).
e2e:   histories/s through the public API including Instrument
construction (IDF parse, table upload), execute and the histogram readback.
roofline: the fused kernels are bound by integer issue (Threefry-4x32-20,
about 150 integer operations per random draw), not by HBM or tensor cores;
achieved = the moderator's Threefry blocks the step needs x ops per block /
kernel time: with the speed look-ahead one per history (its energy) plus
four per history the look-ahead keeps (2.8 % here), else five per history;
peak = the same operation rate measured by a Threefry-only kernel on this
GPU: a lower bound on the issue used.  The DRAM traffic and
the instruction count per history come from the ncu capture recorded in
profiles/ with a hash of the kernel sources; they are reported only when
that hash equals the sources being run.
Beside the headline: the same step without the chopper look-ahead
(fused_without_lookahead), and (one GPU, unless --no-extra) the batched scan of 256
variants (config 3), gradients of a histogram loss (config 4, grads/s) and
the mesh imaging workload (config 5, rays/s with an L2 roofline from the
walk's counted node and triangle reads), the tallies' L2 atomics against a
measured L2-atomic peak, and small-N CUDA-graph replays.
Multi-GPU (torchrun): each rank traces its own 1e8-history slice of one
chunk of N x 1e8 (weak scaling, no collective in the timed region); the
histograms are summed once afterwards.
--impl reference times the reference's own kernels compiled for the host
cores (oracle/refcl, where they build) or else the CPU restatement of them
(the reference's OpenCL runtime path cannot run here), on a bounded sample
with all host threads.
"""
import argparse
import hashlib
import json
import os
import random
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_HIST = 100_000_000
THREEFRY_OPS = 148          # integer operations per Threefry-4x32-20 draw
MCONT_DRAWS = 5             # Threefry blocks the MCont moderator computes per history
CPU_CHUNK = 2_000_000       # histories per chunk of a CPU-baseline step
CPU_SECONDS = 12.0          # CPU work per CPU-baseline step (whole chunks)
NODE_BYTES, TRI_BYTES = 64, 48   # one BVH inner node / triangle as the walk reads them
COUNTERS = os.path.join(HERE, "profiles", "let_like_fused_counters.json")


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=N_HIST)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the config 3/4/5 legs, the atomic roofline and the graph replays")
    p.add_argument("--variants", type=int, default=0,
                   help="batched scan and mesh imaging (--config 3, 5): trace only the "
                        "first N variants (0: all)")
    p.add_argument("--tune", default="auto",
                   help='fused launch config: "auto" (autotuner) or JSON, e.g. {"blocks_per_sm": 3}')
    p.add_argument("--config", type=int, default=2, choices=[2, 3, 4, 5],
                   help="2: LET-like chain (default); 3: batched scan of 256 variants; "
                        "4: gradients of a histogram loss (grads/s); 5: mesh imaging, 360 views")
    return p.parse_args()


def workload_config(n, world, path="fused persistent kernel (plain per-component path "
                                   "reported beside)"):
    return {"workload": "LET-like chain (MCont 40 K, 4 m=2 guides, 5 choppers at Ei 3.7 meV, "
                        "40-line powder, 720x1000 banana histogram)",
            "histories_per_step_per_gpu": n, "global_histories_per_step": n * world,
            "rng": "reference keying (Threefry-4x32-20, one block per draw)",
            "path": path,
            "l2": "flushed between steps (256 MiB write)", "parallelism": "dp%d" % world}


def peaks_file():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# the fused kernels' compile inputs: their translation units, the headers
# those include, the ABI header and the build recipe (flags, instances)
FUSED_SOURCES = ["fused_inst.cu", "fused.cu", "fused_kernel.cuh", "device.cuh", "mesh.cuh",
                 "lookahead.h", "plan.h", "launch.h", "rmath.h", "rconst.h"]


def kernel_source_sha():
    """Hash of the fused kernels' sources and build recipe (the files the
    recorded ncu counters depend on)."""
    h = hashlib.sha256()
    csrc = os.path.join(HERE, "ramp_gb300", "csrc")
    files = [os.path.join(csrc, f) for f in FUSED_SOURCES]
    files += [os.path.join(HERE, "include", "ramp.h"),
              os.path.join(HERE, "ramp_gb300", "build.py")]
    for f in files:
        h.update(os.path.basename(f).encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def profile_counters(tune):
    """Per-history DRAM bytes and warp instructions of the fused launch
    from the recorded ncu captures (one per launch configuration), when one
    was made from these kernel sources with this launch configuration;
    else None with the reason."""
    try:
        with open(COUNTERS) as f:
            c = json.load(f)
    except (OSError, ValueError):
        return None, "no recorded capture"
    sha = kernel_source_sha()
    keys = ("split", "walk", "privatize", "block", "cull")
    why = None
    for cap in c.get("captures", [c]):
        if cap.get("kernel_source_sha") != sha:
            why = "recorded capture is of other kernel sources (%s)" % cap.get("kernel_source_sha")
            continue
        if any(int((tune or {}).get(k, 0)) != int(cap.get("tune", {}).get(k, 0)) for k in keys):
            why = why or "recorded capture is of another launch configuration"
            continue
        return cap, None
    return None, why or "no recorded capture"


def kernels_per_trace(tune):
    """Kernels one fused trace of a chain of the core kinds launches: four
    with the chopper look-ahead from the moderator (the speed table, the
    keep pass, the lean stage A, stage B), three with the mesh walk (stage
    A, the walk, the finish), two with another split (stage A, stage B),
    else one."""
    t = tune or {}
    if int(t.get("walk", 0)) > 0:
        return 3
    if int(t.get("cull", 0)) > 0 and int(t.get("split", 0)) == 0:
        return 4
    return 2 if any(int(t.get(k, 0)) > 0 for k in ("split", "cull")) else 1


# ---------------------------------------------------------------- CPU arm
def cpu_histories_per_s(steps=1, warmup=1, seconds=CPU_SECONDS):
    """The reference's kernels compiled for the host (oracle/refcl, C
    library math), or where they do not build the oracle, on every host
    core over the LET-like chain: one-chunk warm-ups, the last of them
    timed, size each timed step to about ``seconds`` of work in whole
    chunks of CPU_CHUNK histories (bounded memory).  Returns (histories/s
    of the best step, threads, step times, histories per step, kind, what
    ran)."""
    import oracle
    import ramp_gb300 as m
    from oracle import refcl
    from ramp_gb300 import instruments as I
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    threads = os.cpu_count() or 1
    if refcl.available():
        kind, what = "reference", ("the reference's OpenCL kernels compiled for the host "
                                   "(oracle/refcl, C library math), reference sequencing")
        run = lambda n, chunk: refcl.run(inst, n, chunk=chunk, math="libm", threads=threads)
    else:
        kind, what = "port", ("CPU restatement of the reference kernels (reference "
                              "sequencing; the reference's kernels do not build here: %s)"
                              % refcl.unavailable_reason())
        run = lambda n, chunk: oracle.run(inst, n, chunk=chunk, threads=threads)
    pilot = None
    for w in range(max(warmup, 1) + 1):       # the last warm-up chunk is timed
        random.seed(1 + w)
        t0 = time.perf_counter()
        run(CPU_CHUNK, None)
        pilot = time.perf_counter() - t0
    n = max(1, int(round(seconds / max(pilot, 1e-3)))) * CPU_CHUNK
    times = []
    for k in range(steps):
        random.seed(100 + k)
        t0 = time.perf_counter()
        run(n, CPU_CHUNK)
        times.append(time.perf_counter() - t0)
    return n / min(times), threads, times, n, kind, what


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = max(1, a.steps)
    v, threads, times, ns, kind, what = cpu_histories_per_s(steps=steps,
                                                            warmup=max(1, min(a.warmup, 2)))
    sample = ("%d histories of the LET-like chain per step in chunks of %d (a bounded sample, "
              "about %.0f s of CPU work, of the %d-history workload): %s, array-of-structs "
              "records, OpenMP" % (ns, CPU_CHUNK, CPU_SECONDS, a.n, what))
    line = {"metric": "neutron histories/s", "value": v, "unit": "histories/s",
            "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
            "ms_per_step": 1000.0 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(ns, 1, what),
            "cpu_baseline": {"value": v, "unit": "histories/s", "cores": threads,
                             "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "histories/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- clocks
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 7:
                    rows.append(parts)
        os.unlink(self.f.name)
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


# ------------------------------------------------ measurement micro-kernels
def l2_read_peak(lib, dev, mb=32, iters=256):
    """L2 read bandwidth (GB/s) of ramp_debug_l2_peak over an L2-resident
    buffer, best of three."""
    import torch
    from ramp_gb300 import _abi
    buf = torch.ones(mb * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    nth = torch.cuda.get_device_properties(dev).multi_processor_count * 2048
    out = torch.empty(nth, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = _abi.ctypes.c_void_p(stream.cuda_stream)
    best = None
    for k in range(4):
        s, e = _events()
        s.record(stream)
        _abi.check(lib, lib.ramp_debug_l2_peak(buf.data_ptr(), buf.numel(), nth, iters,
                                               out.data_ptr(), sp), "ramp_debug_l2_peak")
        e.record(stream)
        e.synchronize()
        if k:
            gbs = nth * iters * 16 / (s.elapsed_time(e) / 1e3) / 1e9
            best = gbs if best is None else max(best, gbs)
    return best, "ramp_debug_l2_peak: %d threads x %d float4 reads of a %d MB buffer" % (
        nth, iters, mb)


def atomic_peak(lib, dev, n_bins=1 << 20, iters=64):
    """L2 float-atomic adds per second of ramp_debug_atomic_peak, best of
    three."""
    import torch
    from ramp_gb300 import _abi
    bins = torch.zeros(n_bins, dtype=torch.float32, device=dev)
    nth = torch.cuda.get_device_properties(dev).multi_processor_count * 2048
    stream = torch.cuda.current_stream(dev)
    sp = _abi.ctypes.c_void_p(stream.cuda_stream)
    best = None
    for k in range(4):
        s, e = _events()
        s.record(stream)
        _abi.check(lib, lib.ramp_debug_atomic_peak(bins.data_ptr(), n_bins, nth, iters, sp),
                   "ramp_debug_atomic_peak")
        e.record(stream)
        e.synchronize()
        if k:
            r = nth * iters / (s.elapsed_time(e) / 1e3)
            best = r if best is None else max(best, r)
    return best, "ramp_debug_atomic_peak: %d threads x %d float adds into %d bins" % (
        nth, iters, n_bins)


# ------------------------------------------- batched scan and mesh imaging
def batched_workload(config, seed=11):
    """Variants of the batched workloads: (IDF, list of kwargs, counts)."""
    import numpy as np
    from ramp_gb300 import instruments as I
    rng = np.random.default_rng(seed)
    if config == 3:
        ei = np.exp(rng.uniform(np.log(2.0), np.log(20.0), 256))
        slit = rng.uniform(0.010, 0.040, 256)
        counts = np.exp(rng.uniform(np.log(1e5), np.log(4e6), 256)).astype(np.int64)
        kws = [I.let_like_kwargs(Ei=float(e), use_slit=1, slit_w=float(w))
               for e, w in zip(ei, slit)]
        return I.path("let_like.json"), kws, [int(c) for c in counts]
    angles = np.arange(360) * np.pi / 180.0
    kws = [I.mesh_imaging_kwargs(angle=float(t)) for t in angles]
    return I.path("mesh_imaging.json"), kws, [3_000_000] * 360


def mesh_walk_bytes_per_ray(kws, sample=20_000, views=8, seed=3):
    """Algorithmic L2 bytes per ray of the mesh imaging walk: rays drawn as
    the flat moderator draws them (0.06 x 0.06 m source and target, the
    target 1e6 m away), taken into the frame of the mesh (0.5 m downstream,
    rotated about y by each sampled view's angle) and walked through the
    hierarchy the plan builds (ramp_bvh_walk_counts: 64 bytes per inner node
    read, 48 per triangle read)."""
    import numpy as np
    from ramp_gb300 import _abi
    from ramp_gb300.geom.mesh import read_stl_cached
    lib = _abi.load()
    stl = eval(kws[0]["stl_file"])
    pts = np.ascontiguousarray(read_stl_cached(stl), dtype=np.float32)
    rng = np.random.default_rng(seed)
    tot = np.zeros(3, np.int64)
    nr = 0
    for v in np.linspace(0, len(kws) - 1, views).astype(int):
        ang = float(kws[v]["angle"])
        o = np.stack([rng.uniform(-0.03, 0.03, sample), rng.uniform(-0.03, 0.03, sample),
                      np.zeros(sample)], 1)
        t = np.stack([rng.uniform(-0.03, 0.03, sample), rng.uniform(-0.03, 0.03, sample),
                      np.full(sample, 1e6)], 1)
        d = (t - o) / np.linalg.norm(t - o, axis=1, keepdims=True)
        c, s = np.cos(ang), np.sin(ang)
        Ry = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])   # rotation [0, angle, 0]
        p = (o - [0.0, 0.0, 0.5]) @ Ry                        # R^T (o - centre)
        u = d @ Ry
        rays = np.ascontiguousarray(np.concatenate([p, 1000.0 * u], 1), dtype=np.float32)
        out = np.zeros(3, np.int64)
        _abi.check(lib, lib.ramp_bvh_walk_counts(pts.ctypes.data, len(pts), rays.ctypes.data,
                                                 len(rays), out.ctypes.data),
                   "ramp_bvh_walk_counts")
        tot += out
        nr += len(rays)
    return (NODE_BYTES * float(tot[0]) + TRI_BYTES * float(tot[1])) / nr, {
        "nodes_per_ray": float(tot[0]) / nr, "triangles_per_ray": float(tot[1]) / nr,
        "rays_in_mesh_box": float(tot[2]) / nr, "sample_rays": nr}


def measure_batched(config, steps, warmup, tune_arg="auto", variants=0, plain=True):
    """Batched fused path (one launch for all variants) over the full
    workload; the plain path variant after variant on the first 32 variants
    beside it, scaled to all histories."""
    import torch
    import ramp_gb300 as m
    from ramp_gb300.batch import BatchedInstrument
    dev = torch.device("cuda", 0)
    fn, kws, counts = batched_workload(config)
    if variants:            # the first variants only (a small case for profiling)
        kws, counts = kws[:variants], counts[:variants]
    total = sum(counts)
    t0 = time.perf_counter()
    B = BatchedInstrument(fn, kws, ctx=dev)
    setup_s = time.perf_counter() - t0
    if tune_arg == "auto":
        # the autotuner's choice for the first variant (the variants share
        # the component structure)
        from ramp_gb300 import autotune
        tune = {k: v for k, v in autotune.tune(B.instruments[0], rng="reference").items()
                if k in ("block", "blocks_per_sm", "split", "walk", "cull")}
    else:
        tune = json.loads(tune_arg) if tune_arg else None
    for w in range(warmup):
        B.execute(counts, rng="reference", seeds=list(range(len(counts))), tune=tune)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms = []
    for k in range(steps):
        s, e = _events()
        s.record()
        B.execute(counts, rng="reference", seeds=[(k * 7919 + v) % 4097 for v in range(len(counts))],
                  tune=tune)
        e.record()
        e.synchronize()
        ms.append(s.elapsed_time(e))
    clk = clocks.stop()
    out = {"value": total / (statistics.mean(ms) / 1000.0), "ms_per_step": statistics.mean(ms),
           "steps": steps, "warmup": warmup, "variants": len(counts), "histories_per_step": total,
           "tune": tune, "setup_s": setup_s, "clocks": clk,
           "gpu_launches_per_step": kernels_per_trace(tune) *
                                    (sum(1 for c in counts if c > 0)
                                     if int((tune or {}).get("streams", 0)) > 1 else 1)}
    if plain:
        nplain = min(32, len(kws))
        plain_insts = [m.Instrument(fn, dev, **kw) for kw in kws[:nplain]]
        for inst in plain_insts:
            inst.plan()
        torch.cuda.synchronize()
        s, e = _events()
        import random as _r
        s.record()
        for inst, n in zip(plain_insts, counts[:nplain]):
            _r.seed(n)
            inst.execute(n, path="plain")
        e.record()
        e.synchronize()
        plain_ms = s.elapsed_time(e) * total / sum(counts[:nplain])
        out["plain_path_sequential"] = {
            "value": total / (plain_ms / 1000.0), "ms_per_step": plain_ms,
            "sample": "first %d variants, scaled by histories" % nplain}
        out["batched_over_plain"] = out["value"] / out["plain_path_sequential"]["value"]
    return out


def run_batched_config(a):
    import torch
    from ramp_gb300 import build
    build.build()
    torch.cuda.set_device(0)
    r = measure_batched(a.config, a.steps, a.warmup, a.tune, a.variants)
    name = {3: "batched scan: 256 LET-like variants (Ei log-uniform 2-20 meV with matched "
               "chopper phases, slit 10-40 mm, N log-uniform 1e5-4e6), 720x1000 histogram each",
            5: "mesh imaging: 360 views x 3e6 rays through a 200,704-triangle noisy torus "
               "(BVH, watertight chords, mu 0.5/cm), 1024x1024 detector per view"}[a.config]
    line = {"metric": "neutron histories/s", "value": r["value"], "unit": "histories/s",
            "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": name, "variants": r["variants"],
                       "histories_per_step": r["histories_per_step"], "tune": r["tune"],
                       "rng": "reference keying",
                       "path": "batched fused: one launch (two with a split) whose grid "
                               "row v traces variant v"},
            "plain_path_sequential": r.get("plain_path_sequential"),
            "batched_over_plain": r.get("batched_over_plain"),
            "gpu_launches": a.steps * r["gpu_launches_per_step"], "clocks": r["clocks"]}
    print(json.dumps(line), flush=True)


# ------------------------------------------- gradients of a histogram loss
def measure_gradients(steps, warmup, n=10_000_000, fd_check=True):
    """grads/s: forward histogram + loss + adjoint gradient of 22 parameters
    (4 guides x R0, Qc, alpha, m, W; moderator T; powder sigma_abs) on the
    LET-like chain at 1e7 histories; the gradient is also compared with
    central finite differences (common random numbers, step 1e-3)."""
    import numpy as np
    import torch
    import ramp_gb300 as m
    from ramp_gb300 import instruments as I
    from ramp_gb300.diff import DiffChain, LET_LIKE_PARAMS, histogram
    dev = torch.device("cuda", 0)
    inst = m.Instrument(I.path("let_like.json"), dev, **I.let_like_kwargs())
    chain = DiffChain(inst, LET_LIKE_PARAMS, detector="detector")
    theta0 = chain.values()
    r = np.random.default_rng(23)
    chain.set(theta0 * (1.0 + 0.05 * torch.tensor(r.standard_normal(len(theta0)))))
    Ht = chain.forward(n, seed=999).double().clone()

    def step(seed):
        th = theta0.clone().requires_grad_()
        L = ((histogram(chain, th, n, seed).double() - Ht) ** 2).sum()
        L.backward()
        return th.grad

    for w in range(warmup):
        step(10 + w)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms = []
    for k in range(steps):
        s, e = _events()
        s.record()
        step(100 + k)
        e.record()
        e.synchronize()
        ms.append(s.elapsed_time(e))
    clk = clocks.stop()
    out = {"value": 1000.0 / statistics.mean(ms), "unit": "grads/s",
           "ms_per_step": statistics.mean(ms), "steps": steps, "warmup": warmup,
           "histories_per_s_forward_and_adjoint": n / (statistics.mean(ms) / 1000.0),
           "parameters": len(theta0), "histories": n, "clocks": clk}
    if fd_check:
        g = step(1)
        fd = torch.zeros_like(g)
        with torch.no_grad():
            for k in range(len(theta0)):
                h = 1e-3 * float(theta0[k])
                tp, tm = theta0.clone(), theta0.clone()
                tp[k] += h
                tm[k] -= h
                Lp = ((histogram(chain, tp, n, 1).double() - Ht) ** 2).sum()
                Lm = ((histogram(chain, tm, n, 1).double() - Ht) ** 2).sum()
                fd[k] = (Lp - Lm) / (2 * h)
        rel = ((g - fd).abs() / fd.abs().clamp_min(1e-300)).tolist()
        out["gradient_vs_central_fd"] = {
            nm: {"adjoint": float(x), "fd": float(y), "rel_err": float(z)}
            for nm, x, y, z in zip(chain.names, g.tolist(), fd.tolist(), rel)}
        out["max_rel_err_vs_fd"] = max(rel)
    return out


def run_gradients(a):
    import torch
    from ramp_gb300 import build
    build.build()
    torch.cuda.set_device(0)
    r = measure_gradients(a.steps, a.warmup)
    line = {"metric": "grads/s", "value": r["value"], "unit": "grads/s",
            "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "LET-like chain, 1e7 histories, loss sum (H - H*)^2 over the "
                                   "720x1000 detector, 22 parameters, fused forward + adjoint",
                       "histories": r["histories"]},
            "histories_per_s_forward_and_adjoint": r["histories_per_s_forward_and_adjoint"],
            "gpu_launches": a.steps * 3, "clocks": r["clocks"],
            "gradient_vs_central_fd": r.get("gradient_vs_central_fd")}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def graph_small_n(inst_factory, tune, dev, sizes=(100_000, 1_000_000), reps=20):
    """ms per execute() at small N, eager against a CUDA-graph replay of the
    same trace (ramp_gb300.graph), for both paths."""
    import torch
    out = {}
    for path in ("plain", "fused"):
        for n in sizes:
            inst = inst_factory()
            tn = tune if path == "fused" else None
            for _ in range(3):
                inst.execute(n, path=path, tune=tn)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            for _ in range(reps):
                inst.execute(n, path=path, tune=tn)
            torch.cuda.synchronize(dev)
            eager = 1000.0 * (time.perf_counter() - t0) / reps
            g = inst.capture(n, path=path, tune=tn, state=7)
            for _ in range(3):
                g.replay()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            for _ in range(reps):
                g.replay()
            torch.cuda.synchronize(dev)
            graph = 1000.0 * (time.perf_counter() - t0) / reps
            g.check()
            out["%s_%d" % (path, n)] = {"eager_ms": eager, "graph_ms": graph,
                                        "graph_histories_per_s": n / (graph / 1000.0)}
    return out


def issue_roofline(value, clk, dev, counters):
    """Warp instructions issued per second by the fused launch (live
    histories/s x the captured instructions per history) against the
    schedulers' peak at the clock measured during the timed steps."""
    import torch
    if counters is None or not clk.get("sm_mhz"):
        return None
    ipr = counters.get("warp_instructions_per_history")
    if not ipr:
        return None
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak = 4.0 * sms * clk["sm_mhz"] * 1e6
    achieved = value * ipr
    return {"bound": "issue", "achieved": achieved / 1e9, "peak": peak / 1e9,
            "unit": "G warp instructions/s", "frac": achieved / peak,
            "instructions_per_history": ipr,
            "source": "instructions per history from the ncu capture recorded for these kernel "
                      "sources (%s); peak = 4 per SM per cycle x %d SMs x %.0f MHz"
                      % (counters.get("kernel_source_sha"), sms, clk["sm_mhz"])}


def extra_legs(a, lib, dev, peaks):
    """The config 3/4/5 workloads at full size with bounded step counts, and
    the L2 roofline of the mesh walk; each leg is reported on its own and a
    failing leg leaves an error string, never the line."""
    out = {}
    steps, warmup = max(2, min(a.steps, 5)), max(1, min(a.warmup, 3))
    try:
        out["batched_scan"] = dict(measure_batched(3, steps, warmup), unit="histories/s",
                                   workload="config 3: 256 LET-like variants in one launch, "
                                            "720x1000 histogram each")
    except Exception as e:          # a diagnostic leg: never lose the headline
        out["batched_scan"] = {"error": repr(e)[:300]}
    try:
        out["gradients"] = dict(measure_gradients(steps, warmup),
                                workload="config 4: 22 gradients of sum (H - H*)^2, LET-like, "
                                         "1e7 histories, fused forward + adjoint")
    except Exception as e:
        out["gradients"] = {"error": repr(e)[:300]}
    try:
        r = measure_batched(5, max(1, min(a.steps, 2)), 1, plain=False)
        fn, kws, counts = batched_workload(5)
        bpr, detail = mesh_walk_bytes_per_ray(kws)
        l2, l2_how = l2_read_peak(lib, dev)
        rays = r["histories_per_step"]
        achieved = bpr * rays / (r["ms_per_step"] / 1e3) / 1e9
        r.update(unit="rays/s",
                 workload="config 5: 360 views x 3e6 rays through a 200,704-triangle torus, "
                          "1024x1024 detector per view",
                 roofline={"bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s",
                           "frac": achieved / l2 if l2 else None,
                           "algorithmic_bytes_per_ray": bpr, "walk": detail,
                           "peak_source": "measured: " + l2_how,
                           "time": "whole launch (moderator stage and mesh walk) per step"})
        out["mesh_imaging"] = r
    except Exception as e:
        out["mesh_imaging"] = {"error": repr(e)[:300]}
    return out


def main():
    a = args_()
    if a.impl == "reference":
        run_reference(a)
        return
    if a.config in (3, 5):
        run_batched_config(a)
        return
    if a.config == 4:
        run_gradients(a)
        return
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import ramp_gb300 as m
    from ramp_gb300 import _abi, build, instruments as I
    if local == 0:            # one build per node; the other ranks wait for it
        build.build()
    if world > 1:
        dist.barrier()
    lib = _abi.load()
    fn, kw = I.path("let_like.json"), I.let_like_kwargs()
    n = a.n
    shard = (rank, world) if world > 1 else None

    def barrier():
        if world > 1:
            dist.barrier()

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    tune = "auto" if a.tune == "auto" else (json.loads(a.tune) if a.tune else None)
    if tune == "auto":
        from ramp_gb300 import autotune
        tune = autotune.tune(m.Instrument(fn, dev, **kw), rng="reference")

    def timed(inst, path, steps, warmup):
        for w in range(warmup):
            random.seed(10 + w)
            inst.execute(n * world if shard else n, path=path, shard=shard,
                         tune=tune if path == "fused" else None)
        barrier()
        torch.cuda.synchronize()
        ms = []
        for k in range(steps):
            flush.fill_(float(k))
            s, e = _events()
            random.seed(1000 + k)
            s.record()
            inst.execute(n * world if shard else n, path=path, shard=shard,
                         tune=tune if path == "fused" else None)
            e.record()
            e.synchronize()
            ms.append(s.elapsed_time(e))
        torch.cuda.synchronize()
        barrier()
        return ms

    inst = m.Instrument(fn, dev, **kw)
    inst.plan()
    clocks = Clocks(local)
    clocks.start()
    fused_ms = timed(inst, "fused", a.steps, a.warmup)
    clk = clocks.stop()
    plain = m.Instrument(fn, dev, **kw)
    plain_ms = timed(plain, "plain", max(2, a.steps // 2), max(1, min(a.warmup, 2)))

    tot = torch.tensor([sum(fused_ms), sum(plain_ms)], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
        for t in inst.tallies():       # the one exchange step: histogram sum
            dist.all_reduce(t)
    fused_total_ms, plain_total_ms = float(tot[0]), float(tot[1])
    value = world * n * a.steps / (fused_total_ms / 1000.0)
    plain_value = world * n * len(plain_ms) / (plain_total_ms / 1000.0)

    # ---- roofline of the fused kernel: the moderator's Threefry blocks,
    # which every history computes (energy, two position and two target
    # coordinates, cont_mod.cl:36-55; the spin's two draws advance the
    # counter but nothing reads them, and later draws are not counted) ----
    stream = torch.cuda.current_stream(dev)
    nlast = plain.last_chunk
    random.seed(1000 + len(plain_ms) - 1)
    seed_last = plain.source.next_seed()
    # with the speed look-ahead (split at the moderator) every history
    # needs its first block (the energy) and only the kept ones the other
    # four of the moderator
    from ramp_gb300.autotune import speed_kept_fraction
    speed_la = int((tune or {}).get("cull", 0)) > 0 and int((tune or {}).get("split", 0)) == 0
    kept_frac = speed_kept_fraction(plain) if speed_la else 1.0
    draws = float(nlast * (1.0 + (MCONT_DRAWS - 1) * kept_frac))
    # neutrons whose last component is the detector: each adds to both of
    # its histograms (sum p, sum p^2), two float atomics per tally
    det_idx = [c["idx"] for name, c in plain.components() if name == "detector"][0]
    tally_events = int(((plain.state[_abi.LANE["prevcomp"], :nlast] == det_idx) &
                        (plain.state[_abi.LANE["p"], :nlast] != 0)).sum())
    kern = []
    for k in range(3):
        random.seed(1000 + len(plain_ms) - 1)
        s, e = _events()
        rngd = _abi.RampRng()
        tuned = _abi.tune_struct(tune or {})
        s.record(stream)
        rc = lib.ramp_trace_fused(inst.plan(), nlast, nlast, seed_last,
                                  _abi.ctypes.byref(rngd), None, None, _abi.ctypes.byref(tuned),
                                  _abi.ctypes.c_void_p(stream.cuda_stream))
        e.record(stream)
        e.synchronize()
        _abi.check(lib, rc, "ramp_trace_fused")
        kern.append(s.elapsed_time(e))
    kern_ms = statistics.median(kern)
    out = torch.empty(152 * 2048 * 4, dtype=torch.int32, device=dev)
    iters = 256
    sp = _abi.ctypes.c_void_p(stream.cuda_stream)
    for _ in range(2):
        lib.ramp_debug_rng_peak(out.numel(), iters, out.data_ptr(), sp)
    s, e = _events()
    s.record(stream)
    lib.ramp_debug_rng_peak(out.numel(), iters, out.data_ptr(), sp)
    e.record(stream)
    e.synchronize()
    peak_draws_s = out.numel() * iters * 2 / (s.elapsed_time(e) / 1000.0)
    achieved_ops = draws * THREEFRY_OPS / (kern_ms / 1000.0)
    peak_ops = peak_draws_s * THREEFRY_OPS
    inst._check_status(lib, inst.plan())
    counters, stale = profile_counters(tune)
    traffic = (counters["dram_bytes_per_history"] * nlast) if counters else None

    # ---- plain path: its HBM traffic (56 B per generated record, 112 B per
    # record alive at a component's entry, 4 B (die flag) per dead one) ----
    random.seed(1000 + len(plain_ms) - 1)
    from ramp_gb300.autotune import survival
    alive = survival(plain, n, "reference", plain.source.next_seed())
    plain_bytes = 56.0 * n + sum(a_ * 112.0 + (n - a_) * 4.0 for a_ in alive if a_ is not None)
    plain_step_s = plain_total_ms / len(plain_ms) / 1000.0
    peaks = peaks_file()
    hbm_peak = peaks.get("hbm_gbs")
    plain_hbm = {"achieved": plain_bytes / plain_step_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                 "frac": (plain_bytes / plain_step_s / 1e9 / hbm_peak) if hbm_peak else None,
                 "algorithmic_bytes_per_step": plain_bytes,
                 "alive_at_component_entry": alive,
                 "peak_source": "measured (copy bandwidth)" if hbm_peak else None}

    extras = {}
    if world == 1 and int((tune or {}).get("cull", 0)) > 0:
        # ---- the same step without the chopper look-ahead (split where
        # fewer than half the histories are alive), to show what it adds ----
        from ramp_gb300.autotune import split_point
        nl_tune = {k: v for k, v in tune.items() if k not in ("cull", "split")}
        nl_tune["split"] = split_point(plain, alive)
        nl = m.Instrument(fn, dev, **kw)
        nl_ms = []
        for w in range(max(1, min(a.warmup, 2))):
            random.seed(10 + w)
            nl.execute(n, path="fused", tune=nl_tune)
        torch.cuda.synchronize()
        for k in range(max(2, a.steps // 2)):
            flush.fill_(float(k))
            s, e = _events()
            random.seed(1000 + k)
            s.record()
            nl.execute(n, path="fused", tune=nl_tune)
            e.record()
            e.synchronize()
            nl_ms.append(s.elapsed_time(e))
        nl_value = n / (statistics.mean(nl_ms) / 1000.0)
        extras["fused_without_lookahead"] = {
            "value": nl_value, "unit": "histories/s", "ms_per_step": statistics.mean(nl_ms),
            "tune": nl_tune, "fused_over_plain": nl_value / plain_value,
            "note": "the same fused kernels and step with the chopper look-ahead off: every "
                    "history is traced through guide 1, survivors compacted before the first "
                    "component fewer than half of them reach"}
        del nl
    if not a.no_extra and world == 1:
        # ---- tallies: float atomics into L2 against a measured peak ----
        ap, ap_how = atomic_peak(lib, dev)
        atomics = 2.0 * tally_events             # sum p and sum p^2: two adds per event
        extras["atomics"] = {
            "bound": "l2_atomics", "achieved": atomics / (kern_ms / 1e3), "peak": ap,
            "unit": "atomics/s", "frac": atomics / (kern_ms / 1e3) / ap if ap else None,
            "per_launch": atomics,
            "counted": "neutrons of nonzero weight whose last component is the detector "
                       "(%d of %d), "
                       "two float atomic adds each into the sum-p and sum-p^2 histograms, "
                       "before warp aggregation" % (tally_events, nlast),
            "peak_source": "measured: " + ap_how}
        # ---- CUDA graphs at small N ----
        extras["graph_small_n"] = graph_small_n(lambda: m.Instrument(fn, dev, **kw), tune, dev)
        # ---- the same chain fed by the tabulated ISIS moderator (MISIS) ----
        mi = m.Instrument(I.path("let_like_misis.json"), dev, **I.let_like_misis_kwargs())
        misis_ms = []
        for k in range(4):
            random.seed(2000 + k)
            s0, e0 = _events()
            s0.record()
            mi.execute(n, path="fused", tune=tune)
            e0.record()
            e0.synchronize()
            if k > 0:
                misis_ms.append(s0.elapsed_time(e0))
        extras["let_like_misis"] = {
            "value": n / (statistics.mean(misis_ms) / 1000.0), "unit": "histories/s",
            "ms_per_step": statistics.mean(misis_ms),
            "workload": "LET-like chain with the MISIS moderator (synthetic 60 x 100 "
                        "time-energy spectrum), %d histories, fused" % n}

    # ---- end to end through the public API ----
    e2e_steps = 0 if a.no_e2e else max(2, a.steps // 2)
    e2e_ms, h2d, d2h = [], 0, 0
    for k in range(e2e_steps + 1 if e2e_steps else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ei = m.Instrument(fn, dev, **kw)
        random.seed(5000 + k)
        # the launch configuration a user gets from tune="auto" (the
        # autotuner's cached choice for this instrument structure)
        ei.execute(n * world if shard else n, path="fused", shard=shard,
                   tune="auto" if a.tune == "auto" else tune)
        d = ei.data()
        t1 = time.perf_counter()
        if k > 0:
            e2e_ms.append(1000.0 * (t1 - t0))
        keep = []
        src, carr, nc, barr, nb = ei.descriptors(keep)
        h2d = sum(x.nbytes for x in keep) + _abi.ctypes.sizeof(carr) + _abi.ctypes.sizeof(barr)
        d2h = sum(t.numel() * t.element_size() for t in ei.tallies())
        del ei, d
    e2e = world * n / (statistics.mean(e2e_ms) / 1000.0) if e2e_ms else None

    if not a.no_extra and world == 1:
        extras.update(extra_legs(a, lib, dev, peaks))

    if rank != 0:
        return
    cpu = None
    if not a.no_cpu_baseline:
        v, threads, _, ns, kind, what = cpu_histories_per_s(steps=1, warmup=1)
        cpu = {"value": v, "unit": "histories/s", "cores": threads, "kind": kind,
               "sample": "%d LET-like histories in chunks of %d (about %.0f s of CPU work): %s, "
                         "OpenMP, after one-chunk warm-ups" % (ns, CPU_CHUNK, CPU_SECONDS, what)}
    line = {
        "metric": "neutron histories/s", "value": value, "unit": "histories/s",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": fused_total_ms / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(n, world), tune=tune),
        "plain_path": {"value": plain_value, "unit": "histories/s",
                       "ms_per_step": plain_total_ms / len(plain_ms),
                       "bound": "issue (guide bounce loops and Threefry, not HBM)",
                       "hbm": plain_hbm},
        "fused_over_plain": value / plain_value,
        "roofline": {"bound": "issue", "achieved": achieved_ops / 1e9, "peak": peak_ops / 1e9,
                     "unit": "Gop/s", "frac": achieved_ops / peak_ops,
                     "traffic": traffic,
                     "traffic_unit": "DRAM bytes per launch (all its kernels)",
                     "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per "
                                        "history of the capture recorded for these kernel "
                                        "sources, times the histories of the launch"
                                        if counters else stale),
                     "kernel": "k_speed_keep + k_fused" if speed_la else "k_fused", "kernel_ms": kern_ms,
                     "draws_per_launch": draws, "lookahead_kept_fraction": kept_frac,
                     "ops_per_draw": THREEFRY_OPS,
                     "peak_source": "measured: Threefry-only kernel (ramp_debug_rng_peak), "
                                    "%d threads x %d x 2 blocks" % (out.numel(), iters),
                     "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "issue_roofline": issue_roofline(value, clk, dev, counters),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "histories/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "includes": "Instrument(...) parse + plan/table upload, execute(tune=\"auto\", "
                            "cached autotuner choice), data() readback"},
        "gpu_launches": a.steps * kernels_per_trace(tune),
        "clocks": clk,
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
