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
    ("let_like_misis.json", dict(Ei=3.7), 400_000, {"split": 0, "cull": 1}, "reference")])
def test_fused_cull_matches_oracle(cuda_lib, fn, kw, N, tune, rng):
    """Split before guide 1 (stage A: the moderator alone) or before
    chopper 1, with the look-ahead; also with the MISIS source."""
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
    """Variants with different Ei (so different chopper phases): one launch
    with a grid row per variant, or per-variant launches on streams."""
    variants = [I.let_like_kwargs(Ei=3.7), I.let_like_kwargs(Ei=8.0), I.let_like_kwargs(Ei=2.5)]
    counts, seeds = [300_000, 123_457, 200_003], [11, 2222, 4000]
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
