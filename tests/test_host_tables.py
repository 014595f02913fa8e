"""Host-side tables of SPowderN, SIsotropic and the detectors against the reference plugins' own
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


@pytest.mark.parametrize("k", [0, 1])
def test_sqw_tables_equal_the_reference_plugin(k):
    """SIsotropic's S(q,w) parsing and cumulative tables (p(w), p(q|w)) and
    header constants equal the reference plugin's run on the same files
    (tests/golden/sqw_host.npz; the plugin ran with this package's simps in
    place of the SciPy function it calls)."""
    from make_sqw_golden import SQW_FILES
    from ramp_gb300.scat.isotropic import SIsotropic
    g = np.load(os.path.join(GOLD, "sqw_host.npz"))
    p = SIsotropic(fn_inc=os.path.join(GOLD, SQW_FILES[k]), ctx="cpu")
    q, w, pw_cdf, pq_cdf, rho, sa, ss, present = p.channels[1]
    assert present
    for name, ours in (("q", q), ("w", w), ("pw_cdf", pw_cdf), ("pq_cdf", pq_cdf)):
        assert np.array_equal(np.asarray(ours, np.float32).view(np.uint32),
                              g["%s_%d" % (name, k)].view(np.uint32)), name
    assert np.array_equal(np.array([rho, sa, ss], np.float32), g["consts_%d" % k])


def test_simps_is_the_composite_simpson_rule():
    """Odd sample counts: SciPy's composite Simpson rule on an irregular grid;
    even counts: the mean of Simpson on the first n-1 samples plus a final
    trapezoid and a first trapezoid plus Simpson on the last n-1."""
    from scipy.integrate import simpson
    from ramp_gb300.scat.isotropic import simps
    rng = np.random.default_rng(4)
    for n in (3, 5, 9, 21):
        x = np.cumsum(rng.uniform(0.1, 1.0, n))
        y = np.sin(x) + x * x
        assert abs(simps(y, x=x) - simpson(y, x=x)) < 1e-12 * max(1.0, abs(simpson(y, x=x)))
    for n in (4, 6, 10):
        x = np.cumsum(rng.uniform(0.1, 1.0, n))
        y = np.cos(x) + 2 * x
        first = simpson(y[:-1], x=x[:-1]) + 0.5 * (x[-1] - x[-2]) * (y[-1] + y[-2])
        last = simpson(y[1:], x=x[1:]) + 0.5 * (x[1] - x[0]) * (y[0] + y[1])
        assert abs(simps(y, x=x) - 0.5 * (first + last)) < 1e-12 * max(1.0, abs(first))
    assert simps(np.array([2.0]), x=np.array([1.0])) == 0.0
    assert simps(np.array([1.0, 3.0]), x=np.array([0.0, 2.0])) == 4.0
