"""Every instrument shipped with the package parses and traces through the
oracle on the CPU: some tally is nonzero, all are finite, and no status
flag is raised."""
import random

import numpy as np
import pytest

import oracle
import ramp_gb300 as m
from ramp_gb300 import instruments as I

SHIPPED = [
    ("let_like.json", I.let_like_kwargs, 1_000_000),          # 7e-5 reach the detector
    ("let_like_misis.json", I.let_like_misis_kwargs, 1_000_000),
    ("powder_diffractometer.json", I.powder_diffractometer_kwargs, 20_000),
    ("tas_like.json", I.tas_like_kwargs, 20_000),
    ("small_chain.json", I.small_chain_kwargs, 20_000),
    ("mesh_imaging.json", I.mesh_imaging_kwargs, 300),
]


@pytest.mark.parametrize("fn,kw,N", SHIPPED, ids=[s[0] for s in SHIPPED])
def test_shipped_instrument_traces_on_the_oracle(fn, kw, N):
    inst = m.Instrument(I.path(fn), "cpu", **kw())
    random.seed(17)
    r = oracle.run(inst, N)
    assert r.flags == 0
    sums = [float(t.sum()) for t in inst.tallies()]
    assert sums and all(np.isfinite(sums)) and max(sums) > 0
