"""The chopper look-ahead of split fused launches (RampTune.cull) on the
GPU: stage A retires the neutrons that certainly cannot pass the choppers
after the split, and every tally still equals the oracle's (the CPU
restatement traces every neutron through every component) within the
reordering error of float atomics.  The soundness of the bound itself is
checked neutron by neutron on the CPU (test_chopper_lookahead.py)."""
import random

import pytest
import torch

import oracle
import ramp_gb300 as m
from ramp_gb300 import instruments as I
from ramp_gb300.batch import BatchedInstrument

from helpers import tallies_close
from test_gpu_parity import pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fn,kw,N,tune,rng", [
    ("let_like.json", dict(Ei=3.7), 2_000_000, {"split": 0, "cull": 1}, "reference"),
    ("let_like.json", dict(Ei=1.5, use_slit=1, slit_w=0.02), 1_000_000,
     {"split": 0, "cull": 1, "blocks_per_sm": 3}, "native"),
    ("let_like.json", dict(Ei=8.0), 1_000_000, {"split": 1, "cull": 1}, "reference"),
    ("let_like.json", dict(Ei=3.7), 1_000_000,
     {"split": 0, "cull": 1, "block": 128, "blocks_per_sm": 8}, "reference"),
    ("let_like_misis.json", dict(Ei=3.7), 400_000, {"split": 0, "cull": 1}, "reference"),
    ("let_like.json", dict(Ei=3.7), 1_000_003, {"split": 0, "cull": 1}, "reference"),
    ("let_like.json", dict(Ei=3.7), 700, {"split": 0, "cull": 1}, "reference")])
def test_fused_cull_matches_oracle(cuda_lib, fn, kw, N, tune, rng):
    """Split before guide 1 (stage A: the moderator alone) or before
    chopper 1, with the look-ahead; also with the MISIS source, with a
    history count that is not a whole number of work items, and with too
    few histories for the speed table (the keep pass prepares the run
    itself and applies the per-chopper test to every history)."""
    kws = (I.let_like_misis_kwargs if "misis" in fn else I.let_like_kwargs)(**kw)
    gi, ci, r = pair(I.path(fn), kws, N, path="fused", rng=rng, tune=tune)
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob
    assert gi.status_flags == r.flags


def test_fused_cull_with_carry_buffers(cuda_lib):
    """Across chunks the RNG counters are carried per index: the look-ahead
    stands aside (a retired neutron would carry a different counter), and
    the run still equals the oracle's."""
    gi, ci, r = pair(I.path("let_like.json"), I.let_like_kwargs(), 900_000, path="fused",
                     chunk=300_000, tune={"split": 0, "cull": 1})
    tallies_close(gi, ci)


@pytest.mark.parametrize("tune", [{"split": 0, "cull": 1},
                                  {"split": 0, "cull": 1, "streams": 4}])
def test_batched_cull_matches_single_runs(cuda_lib, tune):
    """Variants with different Ei (so different chopper phases), one of
    them too short for a speed table: one launch with a grid row per
    variant, or per-variant launches on streams."""
    variants = [I.let_like_kwargs(Ei=3.7), I.let_like_kwargs(Ei=8.0), I.let_like_kwargs(Ei=2.5),
                I.let_like_kwargs(Ei=5.0)]
    counts, seeds = [300_000, 123_457, 200_003, 900], [11, 2222, 4000, 77]
    B = BatchedInstrument(I.path("let_like.json"), variants, ctx="cuda")
    B.execute(counts, rng="native", seeds=seeds, tune=tune)
    torch.cuda.synchronize()
    for v, (kw, n, seed) in enumerate(zip(variants, counts, seeds)):
        ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
        oracle.run(ci, n, rng_mode=1, variant=v, seeds=[seed])
        tallies_close(B.instruments[v], ci)


def test_cull_without_a_chopper_run_is_refused(cuda_lib):
    inst = m.Instrument(I.path("mesh_imaging.json"), "cuda", **I.mesh_imaging_kwargs(0.37))
    random.seed(3)
    with pytest.raises(RuntimeError, match="cull"):
        inst.execute(10_000, path="fused", tune={"split": 0, "cull": 1})
    with pytest.raises(RuntimeError, match="cull"):
        inst.execute(10_000, path="fused", tune={"cull": 1, "walk": 1})


def test_cull_in_a_captured_graph(cuda_lib):
    """The split launch with the look-ahead replays from a CUDA graph and
    equals the oracle run with the replay's chunk seed."""
    N = 500_000
    kw = I.let_like_kwargs()
    gi = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    g = gi.capture(N, path="fused", tune={"split": 0, "cull": 1}, state=21)
    seeds = g.chunk_seeds(1)
    g.replay()
    g.check()
    ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
    oracle.run(ci, N, seeds=seeds)
    tallies_close(gi, ci)


def test_caller_survivor_buffer_reuse_and_fallback(cuda_lib):
    """Split launches keep their survivors in the caller's buffer
    (ramp_plan_set_survivors) when it is large enough and in one of the
    plan's own otherwise; Instrument grows its buffer with the trace.  Each
    run equals the oracle's."""
    import ctypes
    from ramp_gb300 import _abi
    kw = I.let_like_kwargs()
    tune = {"split": 0, "cull": 1}
    lib = _abi.load()
    assert lib.ramp_survivor_bytes(0) == 0
    assert lib.ramp_survivor_bytes(1) == 128 * 96 + 4
    # a caller buffer far too small for the trace: the plan uses its own
    gi = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    plan = gi.plan()
    small = torch.empty(4096, dtype=torch.uint8, device="cuda")
    assert lib.ramp_plan_set_survivors(plan, ctypes.c_void_p(small.data_ptr()), small.numel()) == 0
    rng = _abi.RampRng(0, 0, 0, 0)
    t = _abi.tune_struct(tune)
    s = torch.cuda.current_stream()
    _abi.check(lib, lib.ramp_trace_fused(plan, 300_000, 300_000, 1234, ctypes.byref(rng), None,
                                         None, ctypes.byref(t), ctypes.c_void_p(s.cuda_stream)),
               "ramp_trace_fused")
    torch.cuda.synchronize()
    ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
    oracle.run(ci, 300_000, seeds=[1234])
    tallies_close(gi, ci)
    # through Instrument: a buffer sized for the trace, larger for a larger one
    gi = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    random.seed(41)
    gi.execute(300_000, path="fused", tune=tune)
    first = gi._surv_buf.numel()
    assert first >= lib.ramp_survivor_bytes(300_000)
    gi.execute(700_000, path="fused", tune=tune)
    torch.cuda.synchronize()
    assert gi._surv_buf.numel() >= lib.ramp_survivor_bytes(700_000) > first
    ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
    random.seed(41)
    oracle.run(ci, 300_000)
    oracle.run(ci, 700_000)
    tallies_close(gi, ci)


@pytest.mark.parametrize("seed,N", [(3, 1_000_000), (6, 1_000_000), (11, 1_000_000),
                                    (20, 1000), (11, 1000)])
def test_fused_cull_on_random_runs_matches_oracle(cuda_lib, tmp_path, seed, N):
    """Random guide and chopper runs (the generator of the CPU soundness
    test) ending in time-of-flight and x-y monitors: the fused launch with
    the look-ahead equals the oracle's tallies (at 1000 histories without
    a speed table: the keep pass prepares the run itself)."""
    import numpy as np
    from test_chopper_lookahead import _random_run
    body, n = _random_run(np.random.default_rng(1000 + seed))
    body += (',"m_tof": {"position": [0.0, 0.0, 60.0], "geom_kernel": {"name": "GPlane", '
             '"width": 1.0, "height": 1.0}, "scat_kernel": {"name": "SDetector1D", '
             '"binning": [0.0, 20.0, 60000.0], "var": "tof", "restore_neutron": true}}'
             ',"m_xy": {"position": [0.0, 0.0, 60.1], "geom_kernel": {"name": "GPlane", '
             '"width": 1.0, "height": 1.0}, "scat_kernel": {"name": "SDetector2D", '
             '"axis1_binning": [-0.2, 0.004, 0.2], "axis2_binning": [-0.2, 0.004, 0.2], '
             '"axis1_var": "x", "axis2_var": "y"}}')
    fn = tmp_path / "rand_mon.json"
    fn.write_text('{"all": {"linear": true,%s}}' % body)
    gi, ci, r = pair(str(fn), {}, N, path="fused", tune={"split": 0, "cull": 1})
    tallies_close(gi, ci)
    assert float(sum(t.abs().sum() for t in ci.tallies())) > 0
