"""SMonochromator and SPowder1: host preparation against the reference's
own plugins (golden values made by tests/golden/make_tas_golden.py), and
the oracle's powder diffractometer against the Bragg law."""
import os
import random

import numpy as np

import ramp_gb300 as m
from ramp_gb300 import _abi, instruments as I
from ramp_gb300.scat.monochromator import gauss_legendre_15

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "tas_host.npz"))


def test_quadrature_tables_match_reference():
    x, w = gauss_legendre_15()
    assert np.array_equal(x, GOLD["gauss_x"].astype(np.float32))
    assert np.array_equal(w, GOLD["gauss_w"].astype(np.float32))


def test_powder1_constants_match_reference():
    for case, want in zip(GOLD["powder1_cases"], GOLD["powder1"]):
        d, pack, vc, sa, mult, dw, f2, dphi = case
        p = m.SPowder1(d_spacing=d, pack=pack, vc=vc, sigma_abs=sa, multiplicity=int(mult),
                       DW=dw, F2=f2, d_phi=dphi)
        got = np.array([p.sigma_scat_v2, p.sigma_abs_v, p.q, p.d_phi], dtype=np.float32)
        assert np.array_equal(got, want)


def test_descriptor_slots():
    inst = m.Instrument(I.path("powder_diffractometer.json"), "cpu",
                        **I.powder_diffractometer_kwargs())
    keep = []
    _, carr, nc, _, _ = inst.descriptors(keep)
    kinds = [carr[j].scat for j in range(nc)]
    assert _abi.S_MONO in kinds and _abi.S_POWDER1 in kinds
    j = kinds.index(_abi.S_MONO)
    assert carr[j].table_len[0] == 15 and carr[j].si[0] == 4


def test_oracle_diffraction_peak_at_bragg_angle():
    """Ei 14.7 meV through the monochromator, d = 2.5 AA powder line: the
    detector peak sits at 2 asin(lambda / 2d)."""
    import oracle
    kw = I.powder_diffractometer_kwargs(Ei=14.7)
    inst = m.Instrument(I.path("powder_diffractometer.json"), "cpu", **kw)
    random.seed(1)
    oracle.run(inst, 200_000)
    h = inst.tallies()[0].numpy()
    assert h.sum() > 0
    lam = 9.04456 / np.sqrt(14.7)
    two_theta = 2 * np.degrees(np.arcsin(lam / (2 * 2.5)))
    peak = -10.0 + 0.1 * (np.argmax(h) + 0.5)
    assert abs(peak - two_theta) < 0.5


def test_oracle_tas_events_follow_the_counter():
    """SRescal keeps the events of the neutrons the final counter flagged;
    with Ef = Ei the energy transfer centres on zero."""
    import oracle
    kw = I.tas_like_kwargs(Ei=5.0, Ef=5.0, dE=0.2)
    inst = m.Instrument(I.path("tas_like.json"), "cpu", **kw)
    random.seed(2)
    r = oracle.run(inst, 200_000)
    comps = dict(inst.components())
    qx, qy, qz, dE, p = comps["Sample"]["scat_kernel"].data()
    hits = int((r.neutrons[:, _abi.LANE["se"]] > 0).sum())
    assert len(qx) == hits > 0
    assert abs(float(np.average(dE, weights=p))) < 0.2
    assert np.all(np.abs(dE) <= 1.1)       # |Ei - Ef| + dE spread of the source and Rescal


def test_rescal_needs_the_plain_path():
    inst = m.Instrument(I.path("tas_like.json"), "cpu", **I.tas_like_kwargs())
    import pytest
    with pytest.raises(ValueError, match="plain"):
        inst.execute(1000, path="fused")


def test_reference_powder_example_peak():
    """The reference's powder example (its parameters in
    tests/golden/powder_reference_example.json): PG(002) at the Bragg angle
    for 3 AA, a d = 3 AA powder line, so the nominal peak is 2theta = 60 deg.
    The fitted centre is 60.05 deg (sigma 1.07 deg) at 4e5 histories: what
    the reference's own present kernels give for its own doc/user/powder.json
    (tests/test_reference_kernels.py runs them); the notebook outputs'
    60.37 deg come from a run that the present kernels and files do not
    reproduce."""
    import oracle
    from scipy.optimize import curve_fit
    h, mn, meV = 6.62607015e-34, 1.674929e-27, 1.602176634e-22
    Ei = 9.09
    lam = h / np.sqrt(2 * mn * Ei * meV) * 1e10
    fn = os.path.join(os.path.dirname(__file__), "golden", "powder_reference_example.json")
    inst = m.Instrument(fn, "cpu", Ei=Ei, Mono_angle=float(np.arcsin(lam / (2 * 3.355))),
                        detector_binning=[50.0, 0.02, 70.0])
    random.seed(7)
    oracle.run(inst, 400_000)
    det = dict(inst.components())["Detector"]["scat_kernel"].data(None)
    x = np.asarray(det[0], dtype=float)
    y = np.asarray(det[1], dtype=float)
    f = lambda t, c, mu, s: c * np.exp(-(t - mu) ** 2 / (2 * s ** 2))
    (c, mu, s), _ = curve_fit(f, x, y, p0=[1e9, 60.0, 2.5])
    assert abs(mu - 60.05) < 0.1 and 0.95 < s < 1.2
