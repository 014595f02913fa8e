#!/usr/bin/env python
"""Benchmark: neutron histories/s of the LET-like chopper-spectrometer chain
(1e8 histories per step, FP32, reference RNG keying) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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
roofline: the fused kernel is bound by integer issue (Threefry-4x32-20,
about 150 integer operations per random draw), not by HBM or tensor cores;
achieved = draws x ops per draw / kernel time, peak = the same operation
rate measured by a Threefry-only kernel on this GPU.
Multi-GPU (torchrun): each rank traces its own 1e8-history slice of one
chunk of N x 1e8 (weak scaling, no collective in the timed region); the
histograms are summed once afterwards.
--impl reference times the CPU restatement of the reference kernels (the
reference's OpenCL path cannot run here) on a bounded sample with all host
threads.
"""
import argparse
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
CPU_CHUNK = 2_000_000       # histories per chunk of a CPU-baseline step
CPU_SECONDS = 12.0          # CPU work per CPU-baseline step (whole chunks)
# DRAM bytes (read + write) of one split launch (stage A + stage B, split
# before chopper 2) per 1e7 histories, from the ncu capture summarised in
# profiles/let_like_fused_split_1e7.md (49 + 83 MB and 121 + 5 MB); the
# traffic grows with the histories traced
FUSED_SPLIT2_DRAM_PER_1E7 = (48.59 + 82.98 + 121.37 + 5.09) * 1e6
# the same capture's issue figures for stage A (88 % of the split launch):
# warp instructions issued on 77.4 % of scheduler cycles, 15.8 of 32 lanes
# active per instruction
FUSED_SPLIT2_STAGE_A_ISSUE = {"issue_active_pct": 77.4, "threads_per_instruction": 15.8}
# warp instructions per history of the split launch in that capture
# (stage A 1.363e9 + stage B 1.136e8 per 1e7 histories): with the live
# throughput this gives the launch's issue rate against the scheduler peak
# (4 warp instructions per SM per cycle)
FUSED_SPLIT2_WARP_INSTR_PER_HISTORY = (1.363146e9 + 1.136426e8) / 1e7


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=N_HIST)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
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


# ---------------------------------------------------------------- CPU arm
def cpu_histories_per_s(steps=1, warmup=1, seconds=CPU_SECONDS):
    """The oracle on every host core over the LET-like chain: one-chunk
    warm-ups, the last of them timed, size each timed step to about
    ``seconds`` of work in whole chunks of CPU_CHUNK histories (bounded
    memory); returns (histories/s of the best step, threads, step times,
    histories per step)."""
    import oracle
    import ramp_gb300 as m
    from ramp_gb300 import instruments as I
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    threads = os.cpu_count() or 1
    pilot = None
    for w in range(max(warmup, 1) + 1):       # the last warm-up chunk is timed
        random.seed(1 + w)
        t0 = time.perf_counter()
        oracle.run(inst, CPU_CHUNK, threads=threads)
        pilot = time.perf_counter() - t0
    n = max(1, int(round(seconds / max(pilot, 1e-3)))) * CPU_CHUNK
    times = []
    for k in range(steps):
        random.seed(100 + k)
        t0 = time.perf_counter()
        oracle.run(inst, n, chunk=CPU_CHUNK, threads=threads)
        times.append(time.perf_counter() - t0)
    return n / min(times), threads, times, n


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = max(1, a.steps)
    v, threads, times, ns = cpu_histories_per_s(steps=steps, warmup=max(1, min(a.warmup, 2)))
    sample = ("%d histories of the LET-like chain per step in chunks of %d (a bounded sample, "
              "about %.0f s of CPU work, of the %d-history workload), CPU restatement of the "
              "reference kernels in reference sequencing (5 passes per component, "
              "array-of-structs records), OpenMP" % (ns, CPU_CHUNK, CPU_SECONDS, a.n))
    line = {"metric": "neutron histories/s", "value": v, "unit": "histories/s",
            "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
            "ms_per_step": 1000.0 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(ns, 1, "CPU restatement, reference sequencing"),
            "cpu_baseline": {"value": v, "unit": "histories/s", "cores": threads,
                             "kind": "port", "sample": sample},
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


def run_batched_config(a):
    """Batched fused path (one launch for all variants) against the plain
    path run variant after variant, on the same histories."""
    import torch
    import ramp_gb300 as m
    from ramp_gb300 import _abi, build
    from ramp_gb300.batch import BatchedInstrument
    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    fn, kws, counts = batched_workload(a.config)
    if a.variants:            # the first variants only (a small case for profiling)
        kws, counts = kws[:a.variants], counts[:a.variants]
    total = sum(counts)
    B = BatchedInstrument(fn, kws, ctx=dev)
    if a.tune == "auto":
        # the autotuner's register cap and split point for the first
        # variant (the variants share the component structure)
        from ramp_gb300 import autotune
        tune = {k: v for k, v in autotune.tune(B.instruments[0], rng="reference").items()
                if k in ("blocks_per_sm", "split", "walk")}
    else:
        tune = json.loads(a.tune) if a.tune else None
    for w in range(a.warmup):
        B.execute(counts, rng="reference", seeds=list(range(len(counts))), tune=tune)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms = []
    for k in range(a.steps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        B.execute(counts, rng="reference", seeds=[(k * 7919 + v) % 4097 for v in range(len(counts))],
                  tune=tune)
        e.record()
        e.synchronize()
        ms.append(s.elapsed_time(e))
    clk = clocks.stop()
    # plain path, variant after variant, on the first 32 variants (each has its
    # own plan; mesh plans build their own BVH), scaled to all histories
    nplain = min(32, len(kws))
    plain_insts = [m.Instrument(fn, dev, **kw) for kw in kws[:nplain]]
    for inst in plain_insts:
        inst.plan()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    import random as _r
    s.record()
    for inst, n in zip(plain_insts, counts[:nplain]):
        _r.seed(n)
        inst.execute(n, path="plain")
    e.record()
    e.synchronize()
    plain_ms = s.elapsed_time(e) * total / sum(counts[:nplain])
    value = total * a.steps / (sum(ms) / 1000.0)
    name = {3: "batched scan: 256 LET-like variants (Ei log-uniform 2-20 meV with matched "
               "chopper phases, slit 10-40 mm, N log-uniform 1e5-4e6), 720x1000 histogram each",
            5: "mesh imaging: 360 views x 3e6 rays through a 200,704-triangle noisy torus "
               "(BVH, watertight chords, mu 0.5/cm), 1024x1024 detector per view"}[a.config]
    line = {"metric": "neutron histories/s", "value": value, "unit": "histories/s", "n_gpus": 1,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": statistics.mean(ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": name, "variants": len(counts), "histories_per_step": total,
                       "tune": tune,
                       "rng": "reference keying",
                       "path": "batched fused: one launch (two with a split) whose grid "
                               "row v traces variant v"},
            "plain_path_sequential": {"value": total / (plain_ms / 1000.0), "ms_per_step": plain_ms,
                                      "sample": "first %d variants, scaled by histories" % nplain},
            "batched_over_plain": (total / (statistics.mean(ms) / 1000.0)) / (total / (plain_ms / 1000.0)),
            "gpu_launches": a.steps * (2 if (int((tune or {}).get("split", 0)) > 0
                                             or int((tune or {}).get("walk", 0)) > 0) else 1) *
                            (sum(1 for c in counts if c > 0)
                             if int((tune or {}).get("streams", 0)) > 1 else 1),
            "clocks": clk}
    print(json.dumps(line), flush=True)


# ------------------------------------------- gradients of a histogram loss
def run_gradients(a, n=10_000_000):
    """grads/s: forward histogram + loss + adjoint gradient of 22 parameters
    (4 guides x R0, Qc, alpha, m, W; moderator T; powder sigma_abs) on the
    LET-like chain at 1e7 histories; the gradient is also compared with
    central finite differences (common random numbers, step 1e-3)."""
    import numpy as np
    import torch
    import ramp_gb300 as m
    from ramp_gb300 import build, instruments as I
    from ramp_gb300.diff import DiffChain, LET_LIKE_PARAMS, histogram
    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
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

    for w in range(a.warmup):
        step(10 + w)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms = []
    for k in range(a.steps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        g = step(100 + k)
        e.record()
        e.synchronize()
        ms.append(s.elapsed_time(e))
    clk = clocks.stop()
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
    table = {nm: {"adjoint": float(x), "fd": float(y), "rel_err": float(z)}
             for nm, x, y, z in zip(chain.names, g.tolist(), fd.tolist(), rel)}
    line = {"metric": "grads/s", "value": 1000.0 / statistics.mean(ms), "unit": "grads/s",
            "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": statistics.mean(ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "LET-like chain, 1e7 histories, loss sum (H - H*)^2 over the "
                                   "720x1000 detector, 22 parameters, fused forward + adjoint",
                       "histories": n},
            "histories_per_s_forward_and_adjoint": n / (statistics.mean(ms) / 1000.0),
            "gpu_launches": a.steps * 2, "clocks": clk,
            "gradient_vs_central_fd": table}
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


def issue_roofline(value, clk, dev, tune):
    """Warp instructions issued per second by the split fused launch (live
    histories/s x the profiled instructions per history) against the
    schedulers' peak at the clock measured during the timed steps."""
    import torch
    if not isinstance(tune, dict) or int(tune.get("split", 0)) != 2 or not clk.get("sm_mhz"):
        return None
    try:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
    except (RuntimeError, AssertionError) as e:     # a diagnostic: never lose the line
        return {"unavailable": str(e)}
    peak = 4.0 * sms * clk["sm_mhz"] * 1e6
    achieved = value * FUSED_SPLIT2_WARP_INSTR_PER_HISTORY
    return {"bound": "issue", "achieved": achieved / 1e9, "peak": peak / 1e9,
            "unit": "G warp instructions/s", "frac": achieved / peak,
            "instructions_per_history": FUSED_SPLIT2_WARP_INSTR_PER_HISTORY,
            "source": "instructions per history from the ncu capture of a 1e7-history "
                      "split launch; peak = 4 per SM per cycle x %d SMs x %.0f MHz"
                      % (sms, clk["sm_mhz"])}


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
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
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

    # ---- roofline of the fused kernel: draws from the plain records ----
    stream = torch.cuda.current_stream(dev)
    recs = plain.state[_abi.LANE["mc"], :plain.last_chunk]
    seed_last = None
    random.seed(1000 + len(plain_ms) - 1)
    seed_last = plain.source.next_seed()
    draws = float((recs.double() - seed_last).sum())
    kern = []
    for k in range(3):
        random.seed(1000 + len(plain_ms) - 1)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rngd = _abi.RampRng()
        tuned = _abi.tune_struct(tune or {})
        s.record(stream)
        rc = lib.ramp_trace_fused(inst.plan(), plain.last_chunk, plain.last_chunk, seed_last,
                                  _abi.ctypes.byref(rngd), None, None, _abi.ctypes.byref(tuned),
                                  _abi.ctypes.c_void_p(stream.cuda_stream))
        e.record(stream)
        e.synchronize()
        _abi.check(lib, rc, "ramp_trace_fused")
        kern.append(s.elapsed_time(e))
    kern_ms = statistics.median(kern)
    out = torch.empty(152 * 2048 * 4, dtype=torch.int32, device=dev)
    iters = 256
    for _ in range(2):
        lib.ramp_debug_rng_peak(out.numel(), iters, out.data_ptr(), _abi.ctypes.c_void_p(stream.cuda_stream))
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    lib.ramp_debug_rng_peak(out.numel(), iters, out.data_ptr(), _abi.ctypes.c_void_p(stream.cuda_stream))
    e.record(stream)
    e.synchronize()
    peak_draws_s = out.numel() * iters * 2 / (s.elapsed_time(e) / 1000.0)
    achieved_ops = draws * THREEFRY_OPS / (kern_ms / 1000.0)
    peak_ops = peak_draws_s * THREEFRY_OPS
    inst._check_status(lib, inst.plan())

    # ---- plain path against HBM: 56 B per generated record, 112 B per
    # record alive at a component's entry, 4 B (die flag) per dead one ----
    random.seed(1000 + len(plain_ms) - 1)
    from ramp_gb300.autotune import survival
    alive = survival(plain, n, "reference", plain.source.next_seed())
    plain_bytes = 56.0 * n + sum(a_ * 112.0 + (n - a_) * 4.0 for a_ in alive if a_ is not None)
    plain_step_s = plain_total_ms / len(plain_ms) / 1000.0
    hbm_peak = peaks_file().get("hbm_gbs")
    plain_roof = {"bound": "hbm", "achieved": plain_bytes / plain_step_s / 1e9,
                  "peak": hbm_peak, "unit": "GB/s",
                  "frac": (plain_bytes / plain_step_s / 1e9 / hbm_peak) if hbm_peak else None,
                  "algorithmic_bytes_per_step": plain_bytes,
                  "alive_at_component_entry": alive,
                  "peak_source": "measured (copy bandwidth)" if hbm_peak else None}

    # ---- CUDA graphs at small N ----
    graphs = graph_small_n(lambda: m.Instrument(fn, dev, **kw), tune, dev)

    # ---- the same chain fed by the tabulated ISIS moderator (MISIS) ----
    mi = m.Instrument(I.path("let_like_misis.json"), dev, **I.let_like_misis_kwargs())
    misis_ms = []
    for k in range(4):
        random.seed(2000 + k)
        s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        mi.execute(n, path="fused", tune=tune)
        e0.record()
        e0.synchronize()
        if k > 0:
            misis_ms.append(s0.elapsed_time(e0))
    misis = {"value": n / (statistics.mean(misis_ms) / 1000.0), "unit": "histories/s",
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

    if rank != 0:
        return
    cpu = None
    if not a.no_cpu_baseline:
        v, threads, _, ns = cpu_histories_per_s(steps=1, warmup=1)
        cpu = {"value": v, "unit": "histories/s", "cores": threads, "kind": "port",
               "sample": "%d LET-like histories in chunks of %d (about %.0f s of CPU work), "
                         "CPU restatement of the reference kernels (reference sequencing), "
                         "OpenMP, after one-chunk warm-ups" % (ns, CPU_CHUNK, CPU_SECONDS)}
    peaks = peaks_file()
    line = {
        "metric": "neutron histories/s", "value": value, "unit": "histories/s",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": fused_total_ms / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(n, world), tune=tune),
        "plain_path": {"value": plain_value, "unit": "histories/s",
                       "ms_per_step": plain_total_ms / len(plain_ms), "roofline": plain_roof},
        "graph_small_n": graphs,
        "let_like_misis": misis,
        "fused_over_plain": value / plain_value,
        "roofline": {"bound": "issue", "achieved": achieved_ops / 1e9, "peak": peak_ops / 1e9,
                     "unit": "Gop/s", "frac": achieved_ops / peak_ops,
                     "traffic": (FUSED_SPLIT2_DRAM_PER_1E7 * plain.last_chunk / 1e7
                                 if int((tune or {}).get("split", 0)) == 2 else None),
                     "traffic_unit": "bytes per launch (stage A + B)",
                     "ncu_stage_a": (FUSED_SPLIT2_STAGE_A_ISSUE
                                     if int((tune or {}).get("split", 0)) == 2 else None),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "1e7-history split launch, scaled by histories",
                     "kernel": "k_fused", "kernel_ms": kern_ms, "draws_per_launch": draws,
                     "ops_per_draw": THREEFRY_OPS,
                     "peak_source": "measured: Threefry-only kernel (ramp_debug_rng_peak), "
                                    "%d threads x %d x 2 blocks" % (out.numel(), iters),
                     "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "issue_roofline": issue_roofline(value, clk, dev, tune),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "histories/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "includes": "Instrument(...) parse + plan/table upload, execute(tune=\"auto\", "
                            "cached autotuner choice), data() readback"},
        "gpu_launches": a.steps * (2 if int((tune or {}).get("split", 0)) > 0 else 1),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
