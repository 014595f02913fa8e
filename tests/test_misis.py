"""MISIS (tabulated ISIS moderator): the spectrum reader and the acceptance
integral against the reference's own reader (golden tables made by
tests/golden/make_misis_golden.py from mcramp/moderator/isis_mod.py), and
the oracle's sampler against properties of the tables."""
import os
import random

import numpy as np
import pytest

import ramp_gb300 as m
from ramp_gb300 import _abi, instruments as I
from ramp_gb300.moderator.isis_mod import read_spectrum, solid_angle_area

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "misis_tables.npz"))
CASES = [(1.1, 9.0, (0.04, 0.09), (0.04, 0.04), 1.7),
         (0.5, 50.0, (0.1, 0.1), (0.03, 0.05), 2.5)]


@pytest.mark.parametrize("k", [0, 1])
def test_reader_matches_reference_tables(k):
    lo, hi, md, td, dist = CASES[k]
    d = read_spectrum(I.ensure_inputs()["spectrum"], lo, hi)
    for name in ("flux", "t_bins", "e_bins", "e_int"):
        g = GOLD["c%d_%s" % (k, name)].astype(np.float32)
        assert d[name].shape == g.shape, name
        assert np.array_equal(d[name], g), name
    assert d["total"] == GOLD["c%d_total" % k]
    assert d["time_offset"] == GOLD["c%d_time_offset" % k]
    assert solid_angle_area(md, td, dist) == GOLD["c%d_str_area" % k]
    nt, ne = GOLD["c%d_sizes" % k]
    assert d["t_bins"].size == nt and d["e_bins"].size == ne
    assert d["flux"].size == (ne - 1) * nt


def test_descriptor_carries_the_tables():
    inst = m.Instrument(I.path("let_like_misis.json"), "cpu", **I.let_like_misis_kwargs())
    src = inst.source.descriptor()
    assert src.kind == _abi.SRC_ISIS
    assert src.table_len[0] == (src.table_len[2] - 1) * src.table_len[1]
    assert src.p[13] == inst.source.str_area and src.p[14] == inst.source.total


def test_oracle_samples_inside_the_tables():
    import oracle
    inst = m.Instrument(I.path("let_like_misis.json"), "cpu", **I.let_like_misis_kwargs())
    random.seed(3)
    r = oracle.run(inst, 100_000)
    rec = r.neutrons
    sp = inst.source.spectrum
    # every history starts alive at the moderator face, with the reference weight
    assert np.all(rec[:, _abi.LANE["mc"]] >= 8)
    v = np.linalg.norm(rec[:, 3:6], axis=1)
    E = (v / 437.393) ** 2
    e_lo, e_hi = float(sp["e_bins"][0]), float(sp["e_bins"][-1])
    # the 7-point Lagrange edge interpolation keeps energies in the table's span
    assert np.nanmin(E) > 0.5 * e_lo and np.nanmax(E) < 2.0 * e_hi
