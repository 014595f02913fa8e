"""CUDA-graph replays of a whole trace (ramp_gb300.graph).

A captured trace draws its chunk seeds on the device; the LCG is restated on
the host (``chunk_seeds``), so every replay can be checked against the oracle
run with the same seeds: plain-path records bit-identical, tallies within
the reordering error of float atomics.
"""
import numpy as np
import pytest
import torch

import oracle
import ramp_gb300 as m
from ramp_gb300 import instruments as I
from ramp_gb300.graph import lcg_seeds

from helpers import _Host, records_equal, tallies_close

pytestmark = pytest.mark.gpu


def test_host_lcg_matches_device(cuda_lib):
    inst = m.Instrument(I.path("small_chain.json"), "cuda", **I.small_chain_kwargs())
    g = inst.capture(1000, path="fused", state=0xdeadbeefcafef00d)
    want, after = lcg_seeds(0xdeadbeefcafef00d, 5)
    got = []
    for _ in range(5):
        g.replay()
        torch.cuda.synchronize()
        got.append(int(g.seed_buf[0]))
    assert got == want
    assert g.state == after
    assert all(0 <= s <= 4096 for s in got)


@pytest.mark.parametrize("path", ["plain", "fused"])
def test_graph_replays_match_oracle(cuda_lib, path):
    N, chunk, reps = 150_000, 65_536, 2
    kw = I.small_chain_kwargs()
    gi = m.Instrument(I.path("small_chain.json"), "cuda", **kw)
    g = gi.capture(N, path=path, chunk=chunk, state=2024)
    assert g.n_chunks == 3
    seeds = g.chunk_seeds(reps)
    for _ in range(reps):
        g.replay()
    g.check()
    ci = m.Instrument(I.path("small_chain.json"), "cpu", **kw)
    for r in range(reps):
        res = oracle.run(ci, N, chunk=chunk, seeds=seeds[r * 3:(r + 1) * 3])
    tallies_close(gi, ci)
    if path == "plain":
        recs, iidx = gi.neutron_state()
        records_equal(recs, res.neutrons)
        assert np.array_equal(iidx, res.iidx)


def test_graph_equals_eager_execute_with_same_seeds(cuda_lib):
    """A replay and an eager execute fed the same chunk seeds agree."""
    N, chunk = 300_000, 100_000
    kw = I.let_like_kwargs()
    a = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    g = a.capture(N, path="fused", chunk=chunk, state=99)
    seeds = iter(g.chunk_seeds(1))
    g.replay()
    g.check()
    b = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    b.source.next_seed = lambda: next(seeds)
    b.execute(N, path="fused", chunk=chunk)
    torch.cuda.synchronize()
    tallies_close(a, _Host(b))


def test_plain_graph_refuses_stale_parameters(cuda_lib):
    from ramp_gb300.diff import DiffChain, LET_LIKE_PARAMS
    inst = m.Instrument(I.path("let_like.json"), "cuda", **I.let_like_kwargs())
    g = inst.capture(10_000, path="plain")
    chain = DiffChain(inst, LET_LIKE_PARAMS, detector="detector")
    chain.set(chain.values())
    with pytest.raises(RuntimeError, match="capture it again"):
        g.replay()


@pytest.mark.parametrize("path", ["plain", "fused"])
def test_gpu_run_resumed_from_a_checkpoint_equals_the_uninterrupted_run(cuda_lib, tmp_path, path):
    """execute() twice, against execute() once, a checkpoint, a fresh
    instrument restored from it and execute() again (the GPU paths)."""
    import random
    kw = I.small_chain_kwargs()
    whole = m.Instrument(I.path("small_chain.json"), "cuda", **kw)
    random.seed(21)
    whole.execute(200_000, path=path)
    whole.execute(200_000, path=path)
    first = m.Instrument(I.path("small_chain.json"), "cuda", **kw)
    random.seed(21)
    first.execute(200_000, path=path)
    first.save_checkpoint(tmp_path / "run.pt")
    random.seed(12345)                   # the process moves on
    resumed = m.Instrument(I.path("small_chain.json"), "cuda", **kw)
    resumed.load_checkpoint(tmp_path / "run.pt")
    resumed.execute(200_000, path=path)
    torch.cuda.synchronize()
    tallies_close(_Host(resumed), _Host(whole))
    assert sum(float(t.sum()) for t in whole.tallies()) > 0
