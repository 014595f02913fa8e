"""Host-side tables of SPowderN against the reference plugin's own
(tests/golden/powdern_host.npz, made by tests/golden/make_powdern_golden.py
from mcramp/scat/powderN.py): q = 2 pi / d, sigma_scat v^2 and
sigma_abs v, bit for bit, including the LET-like chain's 40-line sample."""
import os
import sys

import numpy as np
import pytest

from ramp_gb300.scat.powderN import SPowderN

GOLD = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLD)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_powdern_tables_equal_the_reference_plugin(k):
    from make_powdern_golden import cases
    g = np.load(os.path.join(GOLD, "powdern_host.npz"))
    p = SPowderN(ctx="cpu", **cases()[k])
    assert p.q.dtype == np.float32 and p.sigma_scat_v2.dtype == np.float32
    assert np.array_equal(p.q.view(np.uint32), g["q_%d" % k].view(np.uint32))
    assert np.array_equal(p.sigma_scat_v2.view(np.uint32), g["ssv2_%d" % k].view(np.uint32))
    assert np.float32(p.sigma_abs_v).view(np.uint32) == g["sav_%d" % k].view(np.uint32)[0]
