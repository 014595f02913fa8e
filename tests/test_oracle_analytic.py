"""Closed-form checks of the restated physics, run through the CPU oracle
(the GPU paths equal the oracle bit for bit on records and to float-atomic
order on tallies, tests/test_gpu_parity.py): time of flight to a plane, a
flat moderator spectrum, a guide below its critical angle conserving
weight, and a disk chopper's transmission equal to its open fraction."""
import numpy as np
import pytest
from scipy.stats import chi2

import oracle
import ramp_gb300 as m

SE2V = 437.393   # m/s per sqrt(meV) (consts.h)

PENCIL = """{
  "all": {
    "linear": true,
    "mod": {"source": true, "position": [0, 0, 0],
            "moderator_kernel": {"name": "MFlat", "mod_dim": [$md$, $md$],
                                 "target_dim": [$md$, $md$], "target_dist": 1.0,
                                 "E_min": $e0$, "E_max": $e1$}},
    $middle$
    "mon": {"position": [0, 0, $zm$],
            "geom_kernel": {"name": "GPlane", "width": 0.2, "height": 0.2},
            "scat_kernel": {"name": "SDetector1D", "var": "$var$",
                            "binning": [$b0$, $bs$, $b1$]}}
  }
}
"""

GUIDE = """"guide": {"position": [0, 0, 1.0],
              "geom_kernel": {"name": "GPlane", "width": 0.02, "height": 0.02},
              "scat_kernel": {"name": "SGuide", "w1": 0.02, "h1": 0.02, "w2": 0.02,
                              "h2": 0.02, "l": 6.0, "R0": %s, "Qc": 0.0219,
                              "alpha": 3.0, "m": 2, "W": 0.003}},"""

ABSORBER = """"can": {"position": [0, 0, 1.0],
            "geom_kernel": %s,
            "scat_kernel": {"name": "SPowderN", "d_spacing": [2.0], "pack": 1.0, "vc": 60.0,
                            "sigma_abs": 5.0, "multiplicity": [1], "DW": 1.0, "F2": [0.0],
                            "d_phi": 180.0}},"""

CHOPPER = """"chop": {"position": [0, 0, 1.0],
             "geom_kernel": {"name": "GPlane", "width": 0.6, "height": 0.6},
             "scat_kernel": {"name": "SChopper", "radius": 0.28, "freq": 1884.955592,
                             "n_slits": 6, "jitter": %r, "slit_width": 0.04,
                             "phase": 0.0}},"""


def run(tmp_path, text, N, seed=5, **kw):
    fn = tmp_path / "inst.json"
    fn.write_text(text.replace("$middle$", kw.pop("middle", "")).replace("$var$", kw.pop("var")))
    inst = m.Instrument(str(fn), "cpu", **kw)
    oracle.run(inst, N, seeds=[seed])
    det = dict(inst.components())["mon"]["scat_kernel"]
    return (np.asarray(det.histo, dtype=np.float64), np.asarray(det.histo_err, dtype=np.float64),
            np.asarray(det.axis, dtype=np.float64))


def test_time_of_flight_to_a_plane(tmp_path):
    """A pencil beam of one energy reaches a plane at z = 3 m at t = z / v."""
    E, z = 5.0, 3.0
    h, _, axis = run(tmp_path, PENCIL, 5_000, md=1e-5, e0=E, e1=E, zm=z, var="tof",
                     b0=0.0, bs=1.0, b1=4000.0)
    t_us = z / (SE2V * np.sqrt(E)) * 1e6
    k = int(np.argmax(h))
    assert abs(h.sum() - 1.0) < 2 * 5_000 * 2.0 ** -24   # float32 sums into one bin
    assert k == int(np.floor(t_us))          # floor bins (detector1D.cl:59)


def test_flat_moderator_spectrum(tmp_path):
    """MFlat samples E uniformly: the weighted energy histogram is flat
    (chi-square against a constant, p > 0.001)."""
    h, e, _ = run(tmp_path, PENCIL, 200_000, md=1e-4, e0=2.0, e1=20.0, zm=1.5, var="energy",
                  b0=2.0, bs=0.5, b1=20.0)
    inner = slice(1, -1)                      # edge bins see rounding at E_min and E_max
    hi, ei = h[inner], e[inner]
    mean = hi.mean()
    stat = float(((hi - mean) ** 2 / ei).sum())
    dof = len(hi) - 1
    assert chi2.sf(stat, dof) > 1e-3
    assert abs(h.sum() - 1.0) < 1e-4


@pytest.mark.parametrize("R0", [1.0, 0.5])
def test_guide_below_critical_angle(tmp_path, R0):
    """Divergence up to 5 mrad at 3-3.5 meV keeps q under Qc = 0.0219 1/A, so
    R = R0 at every bounce: with R0 = 1 the weight through a 6 m guide is
    conserved; with R0 = 0.5 the bounces cost weight."""
    h, _, _ = run(tmp_path, PENCIL, 50_000, md=0.005, e0=3.0, e1=3.5, zm=7.05, var="tof",
                  b0=0.0, bs=10.0, b1=20000.0, middle=GUIDE % R0)
    if R0 == 1.0:
        assert abs(h.sum() - 1.0) < 1e-4
    else:
        assert 0.2 < h.sum() < 0.95


def test_chopper_transmission_is_its_open_fraction(tmp_path):
    """With a phase jitter spanning whole slit periods the chopper angle at
    arrival is uniform, so the transmitted fraction is the slit's angular
    width atan(w / r) over the period 2 pi / n_slits."""
    Tg = 2 * np.pi / 6
    N = 100_000
    h, _, _ = run(tmp_path, PENCIL, N, md=1e-5, e0=5.0, e1=5.0, zm=1.5, var="tof",
                  b0=0.0, bs=10.0, b1=20000.0, middle=CHOPPER % float(3 * Tg / 2))
    p = np.arctan2(0.04, 0.28) / Tg
    sigma = np.sqrt(p * (1 - p) / N)
    assert abs(h.sum() - p) < 4 * sigma


@pytest.mark.parametrize("geom", ['{"name": "GCylinderExt", "radius": 0.005, "height": 0.04}',
                                  '{"name": "GSphere", "radius": 0.005}'])
def test_chord_through_an_absorber(tmp_path, geom):
    """A pencil beam through the axis of a cylinder (or the centre of a
    sphere) of radius r crosses a chord of 2 r: with only absorption (all F^2 = 0) the powder kernel
    transmits with probability 1 - p and weight factor 1 - p, where
    p = 1 - exp(-Sigma_abs 2 r) and Sigma_abs = (pack sigma_abs / vc 100)
    2200 / v (powderN.py:65, powderN.cl:40-58), so the weight reaching
    the monitor is (1 - p)^2 per neutron."""
    E, N = 5.0, 100_000
    h, _, _ = run(tmp_path, PENCIL, N, md=1e-5, e0=E, e1=E, zm=1.5, var="tof",
                  b0=0.0, bs=10.0, b1=20000.0, middle=ABSORBER % geom)
    v = SE2V * np.sqrt(E)
    sig = (1.0 * 5.0 / 60.0 * 100.0) * 2200.0 / v
    q = np.exp(-sig * 2 * 0.005)                   # 1 - p
    sigma = q * np.sqrt(q * (1 - q) / N)
    assert abs(h.sum() - q * q) < 4 * sigma
