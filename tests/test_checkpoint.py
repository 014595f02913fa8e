"""Checkpoint and resume between execute() calls (CPU oracle): a run saved
after its first part, restored into a fresh instrument and continued, ends
with the tallies of the uninterrupted run."""
import random

import numpy as np
import pytest
import torch

import oracle
import ramp_gb300 as m
from ramp_gb300 import instruments as I


def make():
    return m.Instrument(I.path("small_chain.json"), "cpu", **I.small_chain_kwargs())


def test_resume_equals_uninterrupted_run(tmp_path):
    whole = make()
    random.seed(5)
    oracle.run(whole, 30_000)
    oracle.run(whole, 30_000)

    first = make()
    random.seed(5)
    oracle.run(first, 30_000)
    first.save_checkpoint(tmp_path / "run.pt")
    random.seed(999)                     # the process moves on
    resumed = make()
    resumed.load_checkpoint(tmp_path / "run.pt")
    oracle.run(resumed, 30_000)
    for a, b in zip(resumed.tallies(), whole.tallies()):
        a, b = a.double().numpy(), b.double().numpy()
        assert np.allclose(a, b, rtol=1e-5, atol=1e-7 * max(np.abs(b).max(), 1e-30))
    assert sum(float(t.sum()) for t in whole.tallies()) > 0


def test_restore_rejects_other_states():
    inst = make()
    with pytest.raises(ValueError, match="not a ramp_gb300 checkpoint"):
        inst.restore({"tallies": []})
    other = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    with pytest.raises(ValueError, match="do not match"):
        inst.restore(other.checkpoint())
