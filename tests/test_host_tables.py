"""Host-side tables of SPowderN and the detectors against the reference plugins' own
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


def test_detector_axes_equal_the_reference_plugins():
    """Bin counts, the 1D axis and the 2D coordinate grids of SDetector1D
    and SDetector2D equal the reference plugins' (tests/golden/detector_axes.npz,
    made by tests/golden/make_detector_golden.py)."""
    from make_detector_golden import BINNINGS_1D, BINNINGS_2D
    from ramp_gb300.scat.detector1D import SDetector1D
    from ramp_gb300.scat.detector2D import SDetector2D
    g = np.load(os.path.join(GOLD, "detector_axes.npz"))
    for k, b in enumerate(BINNINGS_1D):
        det = SDetector1D(binning=b, var="theta", ctx="cpu")
        assert np.array_equal(np.asarray(det.axis), g["axis1d_%d" % k]), b
    for k, (b1, b2) in enumerate(BINNINGS_2D):
        det = SDetector2D(axis1_binning=b1, axis2_binning=b2, axis1_var="theta",
                          axis2_var="tof", ctx="cpu")
        assert [int(det.axis1_num_bins), int(det.axis2_num_bins)] == list(g["n_%d" % k])
        assert np.array_equal(det.X, g["X_%d" % k]) and np.array_equal(det.Y, g["Y_%d" % k])
