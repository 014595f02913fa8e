"""Edge cases of the reference kernels that the restatement bounds, run
through the CPU oracle: a powder whose lines all have F^2 = 0 (the
reference's line walk, powderN.cl:77-85, never reaches a line: the sum of
the line cross-sections is 0) and a guide whose walls reflect nothing."""
import numpy as np
import pytest

import oracle
import ramp_gb300 as m

SAMPLE_IDF = """{
  "all": {
    "linear": true,
    "mod": {"source": true, "position": [0, 0, 0],
            "moderator_kernel": {"name": "MFlat", "mod_dim": [0.005, 0.005],
                                 "target_dim": [0.005, 0.005], "target_dist": 1.0,
                                 "E_min": 3.0, "E_max": 30.0}},
    "sample": {"position": [0, 0, 1.0], "restore_neutron": true,
               "geom_kernel": {"name": "GCylinderExt", "radius": 0.005, "height": 0.04},
               "scat_kernel": {"name": "SPowderN", "d_spacing": [3.1, 2.4, 1.9],
                               "pack": 1.0, "vc": 60.0, "sigma_abs": $sa$,
                               "multiplicity": [6, 8, 12], "DW": 1.0,
                               "F2": [$f2$, $f2$, $f2$], "d_phi": 180.0}},
    "det": {"position": [0, 0, 1.0],
            "geom_kernel": {"name": "GBanana", "radius": 0.5, "height": 0.2,
                            "mintheta": -3.14, "maxtheta": 3.14},
            "scat_kernel": {"name": "SDetector1D", "var": "theta", "binning": [-180, 1, 180]}}
  }
}
"""

GUIDE_IDF = """{
  "all": {
    "linear": true,
    "mod": {"source": true, "position": [0, 0, 0],
            "moderator_kernel": {"name": "MFlat", "mod_dim": [0.03, 0.03],
                                 "target_dim": [0.02, 0.02], "target_dist": 1.0,
                                 "E_min": 2.0, "E_max": 20.0}},
    "guide": {"position": [0, 0, 1.0],
              "geom_kernel": {"name": "GPlane", "width": 0.02, "height": 0.02},
              "scat_kernel": {"name": "SGuide", "w1": 0.02, "h1": 0.02, "w2": 0.02,
                              "h2": 0.02, "l": 2.0, "R0": $r0$, "Qc": 0.0219,
                              "alpha": 3.0, "m": 2, "W": 0.003}},
    "mon": {"position": [0, 0, 3.01],
            "geom_kernel": {"name": "GPlane", "width": 0.1, "height": 0.1},
            "scat_kernel": {"name": "SDetector1D", "var": "tof", "binning": [0, 10, 20000]}}
  }
}
"""


def instrument(tmp_path, text, **kw):
    fn = tmp_path / "inst.json"
    fn.write_text(text)
    return m.Instrument(str(fn), "cpu", **kw)


def det_sum(inst, name):
    return float(np.asarray(dict(inst.components())[name]["scat_kernel"].histo).sum())


@pytest.mark.parametrize("sa", [0.0, 5.0])
def test_powder_with_no_line_cross_section_terminates(tmp_path, sa):
    """All F^2 = 0: every neutron transmits (sigma_abs = 0) or, scattered,
    carries weight 0 (sigma_abs > 0); the run ends and tallies nothing
    scattered."""
    inst = instrument(tmp_path, SAMPLE_IDF, f2=0.0, sa=sa)
    r = oracle.run(inst, 20_000, seeds=[7])
    assert r.flags == 0
    h = np.asarray(dict(inst.components())["det"]["scat_kernel"].histo)
    assert np.isfinite(h).all()
    live = r.neutrons[:, 15] == 0
    if sa == 0.0:
        # p_inter = 0: the transmit branch keeps every neutron's weight
        assert np.all(r.neutrons[live, 9] > 0)
    else:
        assert np.all(r.neutrons[live, 9] >= 0)


def test_powder_with_lines_scatters(tmp_path):
    inst = instrument(tmp_path, SAMPLE_IDF, f2=50.0, sa=1.0)
    oracle.run(inst, 20_000, seeds=[7])
    assert det_sum(inst, "det") > 0


@pytest.mark.parametrize("r0", [0.0, 0.99])
def test_guide_without_reflection_passes_only_straight_neutrons(tmp_path, r0):
    """R0 = 0: every wall bounce sets the weight to 0, so only neutrons that
    cross the guide without touching a wall reach the monitor with weight;
    R0 = 0.99 lets reflected ones through too."""
    inst = instrument(tmp_path, GUIDE_IDF, r0=r0)
    r = oracle.run(inst, 20_000, seeds=[3])
    assert r.flags == 0
    total = det_sum(inst, "mon")
    assert total > 0
    if r0 == 0.0:
        ref = instrument(tmp_path, GUIDE_IDF, r0=0.99)
        oracle.run(ref, 20_000, seeds=[3])
        assert total < det_sum(ref, "mon")


# ----------------------------------------------------------------- GPU
def _gpu_pair(tmp_path, text, N, path, **kw):
    import random
    import torch
    fn = tmp_path / "inst.json"
    fn.write_text(text)
    gi = m.Instrument(str(fn), "cuda", **kw)
    random.seed(99)
    gi.execute(N, path=path)
    torch.cuda.synchronize()
    ci = m.Instrument(str(fn), "cpu", **kw)
    random.seed(99)
    r = oracle.run(ci, N)
    return gi, ci, r


@pytest.mark.gpu
@pytest.mark.parametrize("text,kw", [(SAMPLE_IDF, dict(f2=0.0, sa=5.0)),
                                     (GUIDE_IDF, dict(r0=0.0))],
                         ids=["powder_without_line_cross_section", "guide_without_reflection"])
def test_edge_instruments_match_oracle_on_the_gpu(cuda_lib, tmp_path, text, kw):
    from helpers import records_equal, tallies_close
    gi, ci, r = _gpu_pair(tmp_path, text, 30_000, "plain", **kw)
    recs, iidx = gi.neutron_state()
    records_equal(recs, r.neutrons)
    assert np.array_equal(iidx, r.iidx)
    tallies_close(gi, ci)
    gf, cf, _ = _gpu_pair(tmp_path, text, 30_000, "fused", **kw)
    tallies_close(gf, cf)
