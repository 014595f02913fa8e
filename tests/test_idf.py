"""Instrument definition files: the reference's substitution, comment,
disable, relative-frame, index and block rules (mcramp.py:35-116, 254-355),
checked on the host without a GPU."""
import json

import numpy as np
import pytest

import ramp_gb300 as m
from ramp_gb300 import _abi
from ramp_gb300.instrument import frame_rotate

IDF = """// test instrument
{
  "primary": {
    "linear": true,
    "mod": {"source": true, "position": [0, 0, 0],
            "moderator_kernel": {"name": "MFlat", "mod_dim": [0.01, 0.01],
                                 "target_dim": [0.01, 0.01], "target_dist": $dist$,
                                 "E_min": $2*E$, "E_max": $xx$}},
    "arm": {"position": [0, 0, 1.0], "rotation": [0.0, $ang$, 0.0],
            "geom_kernel": {"name": "GArm"}, "scat_kernel": {"name": "SArm"}},
    "off": {"disable": $skip$, "position": [0, 0, 2.0],
            "geom_kernel": {"name": "GArm"}, "scat_kernel": {"name": "SArm"}},
    "slit": {"position": [0.1, 0.0, 0.5], "relative": "arm", "restore_neutron": true,
             "geom_kernel": {"name": "GPlane", "width": 0.02, "height": 0.03,
                             "orientation": "yz"},
             "scat_kernel": {"name": "SArm"}}   // trailing comment
  },
  "environment": {
    "linear": false,
    "multi": 3,
    "can": {"position": [0, 0, 3.0],
            "geom_kernel": {"name": "GSphere", "radius": 0.01},
            "scat_kernel": {"name": "SBeamstop"}}
  },
  "tail": {
    "det": {"position": [0, 0, 4.0],
            "geom_kernel": {"name": "GPlane", "width": 0.1, "height": 0.1},
            "scat_kernel": {"name": "SDetector1D", "var": "tof", "binning": [0, 10, 1000]}}
  }
}
"""


def make(tmp_path, **kw):
    fn = tmp_path / "inst.json"
    fn.write_text(IDF)
    args = dict(dist=1.5, E=2.5, x=3, xx=7, ang=0.3, skip=1)
    args.update(kw)
    return m.Instrument(str(fn), "cpu", **args)


def test_substitution_and_comments(tmp_path):
    inst = make(tmp_path)
    src = inst.source
    assert src.target_dist == np.float32(1.5)
    assert src.E_min == np.float32(5.0)
    # the reference substitutes variable names as substrings, in keyword
    # order: with x before xx, the token "xx" becomes "33"
    assert src.E_max == np.float32(33.0)


def test_substring_rule_depends_on_keyword_order(tmp_path):
    fn = tmp_path / "inst.json"
    fn.write_text(IDF)
    inst = m.Instrument(str(fn), "cpu", dist=1.5, E=2.5, xx=7, x=3, ang=0.3, skip=1)
    assert inst.source.E_max == np.float32(7.0)


def test_disable_and_indices(tmp_path):
    names = [n for n, _ in make(tmp_path).components()]
    assert names == ["arm", "slit", "can", "det"]
    comps = dict(make(tmp_path).components())
    # the source takes index 1; disabled components take none
    assert [comps[n]["idx"] for n in names] == [2, 3, 4, 5]
    names2 = [n for n, _ in make(tmp_path, skip=0).components()]
    assert names2 == ["arm", "off", "slit", "can", "det"]


def test_relative_frame(tmp_path):
    comps = dict(make(tmp_path).components())
    arm, slit = comps["arm"], comps["slit"]
    want = np.add(frame_rotate([0.1, 0.0, 0.5], [0.0, 0.3, 0.0]), [0.0, 0.0, 1.0])
    assert np.allclose(slit["pos"], want)
    assert np.allclose(slit["rot"], arm["rot"])
    assert slit["restore_neutron"] == 1


def test_blocks_and_descriptor_slots(tmp_path):
    inst = make(tmp_path)
    src, carr, nc, barr, nb = inst.descriptors([])
    assert nc == 4 and nb == 3
    blocks = [(barr[k].first, barr[k].count, barr[k].linear, barr[k].multi) for k in range(nb)]
    assert blocks == [(0, 2, 1, 1), (2, 1, 0, 3), (3, 1, 1, 1)]
    assert carr[1].geom == _abi.G_PLANE and carr[1].gi[0] == 1 and carr[1].restore == 1
    assert carr[2].geom == _abi.G_SPHERE and carr[2].scat == _abi.S_BEAMSTOP
    assert src.kind == _abi.SRC_FLAT


def test_execute_without_a_gpu_fails_loudly(tmp_path):
    inst = make(tmp_path)
    with pytest.raises(RuntimeError):
        inst.execute(10)


def test_parses_equal_the_reference_parser():
    """Component order, indices, lab positions and rotations (float32),
    restore flags and block structure of three instrument files equal the
    reference parser's own (tests/golden/idf_parse.json, made by
    tests/golden/make_idf_golden.py running mcramp.Instrument)."""
    import os
    import sys
    gold_dir = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, gold_dir)
    from make_idf_golden import cases
    gold = json.load(open(os.path.join(gold_dir, "idf_parse.json")))
    for key, fn, kw in cases():
        inst = m.Instrument(fn, "cpu", **kw)
        want = gold[key]
        assert [b.linear for b in inst.blocks] == [b["linear"] for b in want]
        for b, wb in zip(inst.blocks, want):
            got = list(b.components.items())
            assert [n for n, _ in got] == [c["name"] for c in wb["components"]]
            for (name, c), w in zip(got, wb["components"]):
                assert c["idx"] == w["idx"], (key, name)
                assert np.array_equal(np.asarray(c["pos"], np.float32),
                                      np.asarray(w["pos"], np.float32)), (key, name)
                assert np.array_equal(np.asarray(c["rot"], np.float32),
                                      np.asarray(w["rot"], np.float32)), (key, name)
                assert int(c["restore_neutron"]) == w["restore"], (key, name)


def test_reference_examples_parse_and_trace(tmp_path, monkeypatch):
    """The reference's own example instruments (examples/LET.json with the
    MISIS moderator and its spectrum file, examples/TAS.json with relative
    frames and SRescal, the MCPL examples), read unchanged from a checkout
    with the parameters of its scripts: our parse equals the reference
    parser's (run in a subprocess with stand-ins; where that fails, ours
    fails the same way), and the chains without host components trace
    through the oracle.  Skipped without a checkout."""
    import os
    import subprocess
    import sys
    import oracle
    from oracle import build as ob
    ex = os.path.join(ob.REFERENCE, "examples")
    if not os.path.isdir(ex):
        pytest.skip("reference checkout not available")
    gold_dir = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, gold_dir)
    from make_idf_golden import example_cases
    out = tmp_path / "examples_parse.json"
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    subprocess.run([sys.executable, os.path.join(gold_dir, "make_idf_golden.py"), "--examples",
                    ob.REFERENCE, str(out)], cwd=ex, env=env, check=True)
    want = json.load(open(out))
    monkeypatch.chdir(ex)
    for key, fn, kw in example_cases():
        if isinstance(want[key], dict):            # the reference parser fails on it
            with pytest.raises(Exception) as info:
                m.Instrument(fn, "cpu", **kw)
            assert type(info.value).__name__ == want[key]["error"]
            continue
        inst = m.Instrument(fn, "cpu", **kw)
        assert [b.linear for b in inst.blocks] == [b["linear"] for b in want[key]]
        for b, wb in zip(inst.blocks, want[key]):
            got = list(b.components.items())
            assert [n for n, _ in got] == [c["name"] for c in wb["components"]]
            for (name, c), w in zip(got, wb["components"]):
                assert c["idx"] == w["idx"], (key, name)
                assert np.array_equal(np.asarray(c["pos"], np.float32),
                                      np.asarray(w["pos"], np.float32)), (key, name)
                assert np.array_equal(np.asarray(c["rot"], np.float32),
                                      np.asarray(w["rot"], np.float32)), (key, name)
                assert int(c["restore_neutron"]) == w["restore"], (key, name)
        if inst.host_components():                  # MCPL files: traced on the GPU only
            continue
        r = oracle.run(inst, 20_000, seeds=[11])
        assert r.flags == 0
        sums = [float(t.sum()) for t in inst.tallies()]
        assert all(np.isfinite(sums)) and max(sums) > 0, key
