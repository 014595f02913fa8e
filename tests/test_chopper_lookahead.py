"""The chopper look-ahead of split fused launches (RampTune.cull,
ramp_gb300/csrc/lookahead.h), on the CPU.

Soundness: the bound is evaluated on each neutron's state after the
moderator (the oracle's records of a moderator + arm chain) and compared
with what the oracle's trace of moderator -> guide -> chopper -> chopper
does with the same neutrons (same keys, same seeds): no neutron that
passes both choppers (mcramp/scat/chopper.cl:4-59) may be retired.
Efficiency: the bound retires most of those that do not pass.  The run
detection (ramp_chopper_run) accepts only on-axis, unrotated, straight
runs."""
import ctypes

import numpy as np
import pytest

import oracle
import ramp_gb300 as m
from ramp_gb300 import _abi

MOD = '''
    "mod": {"source": true, "position": [0.0, 0.0, 0.0],
      "moderator_kernel": {"name": "MCont", "mod_dim": [0.1, 0.1], "target_dim": [0.04, 0.04],
        "target_dist": 1.7, "E_min": 1.1, "E_max": 9.0, "T1": 40.0, "I1": 1.0,
        "T2": 40.0, "I2": 0.0, "T3": 40.0, "I3": 0.0}}'''

RUN = '''
    "guide1": {"position": [0.0, 0.0, 1.7],
      "geom_kernel": {"name": "GPlane", "width": 0.04, "height": 0.04},
      "scat_kernel": {"name": "SGuide", "w1": 0.04, "h1": 0.04, "w2": $gw2$, "h2": 0.04,
        "l": 6.05, "R0": 0.99, "Qc": 0.0219, "alpha": 3.0, "m": 2, "W": 0.003}},
    "chopper1": {"position": [0.0, $cy$, 7.8],
      "geom_kernel": {"name": "GPlane", "width": 0.6, "height": 0.6},
      "scat_kernel": {"name": "SChopper", "radius": 0.28, "freq": 1884.955592, "n_slits": 6,
        "jitter": 7e-07, "slit_width": 0.04, "phase": $7.80 / (437.393*Ei**0.5)$}},
    "chopper2": {"position": [0.0, 0.0, 8.4],
      "geom_kernel": {"name": "GPlane", "width": 0.6, "height": 0.6},
      "scat_kernel": {"name": "SChopper", "radius": 0.28, "freq": 62.831853, "n_slits": 1,
        "jitter": 7e-07, "slit_width": 0.04, "phase": $8.40 / (437.393*Ei**0.5)$}}'''

RUN2 = '''
    "guide2": {"position": [0.0, 0.0, 8.45],
      "geom_kernel": {"name": "GPlane", "width": 0.04, "height": 0.04},
      "scat_kernel": {"name": "SGuide", "w1": 0.04, "h1": 0.04, "w2": 0.04, "h2": 0.04,
        "l": 3.3, "R0": 0.99, "Qc": 0.0219, "alpha": 3.0, "m": 2, "W": 0.003}},
    "chopper3": {"position": [0.0, 0.0, 11.8],
      "geom_kernel": {"name": "GPlane", "width": 0.6, "height": 0.6},
      "scat_kernel": {"name": "SChopper", "radius": 0.28, "freq": 942.477796, "n_slits": 2,
        "jitter": 7e-07, "slit_width": 0.04, "phase": $11.80 / (437.393*Ei**0.5)$}},
    "guide3": {"position": [0.0, 0.0, 11.85],
      "geom_kernel": {"name": "GPlane", "width": 0.03, "height": 0.04},
      "scat_kernel": {"name": "SGuide", "w1": 0.03, "h1": 0.04, "w2": 0.03, "h2": 0.04,
        "l": 3.8, "R0": 0.99, "Qc": 0.0219, "alpha": 3.0, "m": 2, "W": 0.003}},
    "chopper4": {"position": [0.0, 0.0, 15.7],
      "geom_kernel": {"name": "GPlane", "width": 0.6, "height": 0.6},
      "scat_kernel": {"name": "SChopper", "radius": 0.28, "freq": 942.477796, "n_slits": 6,
        "jitter": 7e-07, "slit_width": 0.04, "phase": $15.70 / (437.393*Ei**0.5)$}}'''

ARM = '''
    "arm": {"position": [0.0, 0.0, 0.0], "geom_kernel": {"name": "GArm"},
      "scat_kernel": {"name": "SArm"}}'''


def instrument(tmp_path, name, body, **kw):
    fn = tmp_path / name
    fn.write_text('{"all": {"linear": true,%s}}' % body)
    return m.Instrument(str(fn), "cpu", **kw)


def run_length(inst, k):
    keep = []
    _, carr, nc, barr, nb = inst.descriptors(keep)
    return _abi.load().ramp_chopper_run(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, k)


def culled(inst, k, records):
    keep = []
    _, carr, nc, barr, nb = inst.descriptors(keep)
    rec = np.ascontiguousarray(records, dtype=np.float32)
    out = np.zeros(len(rec), np.uint8)
    lib = _abi.load()
    rc = lib.ramp_debug_chopper_cull(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, k,
                                     rec.ctypes.data, len(rec), out.ctypes.data)
    _abi.check(lib, rc, "ramp_debug_chopper_cull")
    return out.astype(bool)


def speed_culled(inst, k, n, seed):
    """The speed-only bound (ramp_debug_speed_cull) for neutrons 0..n-1 of
    a reference-keyed run with this chunk seed: neutron i's energy draw is
    the Threefry word of counter seed and index i."""
    keep = []
    src, carr, nc, barr, nb = inst.descriptors(keep)
    words = np.ascontiguousarray(oracle.threefry(np.full(n, seed, np.uint32),
                                                 np.arange(n, dtype=np.uint32)))
    p = np.ascontiguousarray(np.array(src.p[0:7], dtype=np.float32))
    out = np.zeros(n, np.uint8)
    check = np.zeros(2, np.int64)
    lib = _abi.load()
    rc = lib.ramp_debug_speed_cull(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, k,
                                   p.ctypes.data, words.ctypes.data, n, out.ctypes.data,
                                   check.ctypes.data)
    _abi.check(lib, rc, "ramp_debug_speed_cull")
    assert check[1] == 0          # the speed table agrees with the per-chopper test
    return out.astype(bool)


def test_speed_table_equals_the_per_chopper_test():
    """The cells of the speed table (lookahead.h) decide most energy draws,
    and every draw they decide gets the per-chopper test's answer, also for
    the first and last words of every cell and their neighbours."""
    import ramp_gb300 as m
    from ramp_gb300 import instruments as I
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    src, carr, nc, barr, nb = inst.descriptors([])
    rng = np.random.default_rng(5)
    rand = rng.integers(0, 1 << 32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    first = (np.arange(4096, dtype=np.uint64) << 19).astype(np.uint32)
    edges = [first, first + np.uint32(1), first + np.uint32(64), first - np.uint32(1),
             first - np.uint32(64), first | np.uint32(1 << 31)]
    words = np.ascontiguousarray(np.concatenate([rand] + edges), dtype=np.uint32)
    p = np.ascontiguousarray(np.array(src.p[0:7], dtype=np.float32))
    out = np.zeros(len(words), np.uint8)
    check = np.zeros(2, np.int64)
    lib = _abi.load()
    _abi.check(lib, lib.ramp_debug_speed_cull(ctypes.addressof(carr), nc, ctypes.addressof(barr),
                                              nb, 0, p.ctypes.data, words.ctypes.data,
                                              len(words), out.ctypes.data, check.ctypes.data),
               "ramp_debug_speed_cull")
    assert check[1] == 0
    assert check[0] > 0.99 * len(words)
    assert 0.01 < 1.0 - out[:1_000_000].mean() < 0.05     # about 2.8 % kept


@pytest.mark.parametrize("Ei", [1.5, 3.7, 8.0])
def test_lookahead_never_retires_a_neutron_that_passes(tmp_path, Ei):
    N = 400_000
    kw = dict(Ei=Ei, gw2=0.04, cy=0.0)
    full = instrument(tmp_path, "run.json", MOD + "," + RUN, **kw)
    arm = instrument(tmp_path, "arm.json", MOD + "," + ARM, **kw)
    assert run_length(full, 0) == 3          # the guide and both choppers
    seeds = [1234]
    after_mod = oracle.run(arm, N, seeds=seeds).neutrons
    traced = oracle.run(full, N, seeds=seeds).neutrons
    passed = traced[:, 15] == 0.0
    # the same neutrons: a neutron through both choppers drew twice more
    assert np.array_equal(after_mod[passed, 11] + 2, traced[passed, 11])
    cut = culled(full, 0, after_mod)
    assert passed.sum() > 100
    assert not (cut & passed).any(), "a neutron that passes the choppers was retired"
    # most of those that do not pass are retired before the guide
    assert cut.sum() >= 0.8 * (~passed).sum()
    # the speed-only bound retires a subset of those, and no passing one
    scut = speed_culled(full, 0, N, seeds[0])
    assert not (scut & passed).any(), "the speed bound retired a neutron that passes"
    assert scut.sum() > 0.3 * (~passed).sum()


@pytest.mark.parametrize("Ei", [2.0, 3.7])
def test_lookahead_through_several_guides_never_retires_a_neutron_that_passes(tmp_path, Ei):
    """The run guide, chopper, chopper, guide, chopper, guide (narrower than
    the ones before it, so some neutrons miss its entrance), chopper."""
    N = 400_000
    kw = dict(Ei=Ei, gw2=0.04, cy=0.0)
    full = instrument(tmp_path, "run2.json", MOD + "," + RUN + "," + RUN2, **kw)
    arm = instrument(tmp_path, "arm.json", MOD + "," + ARM, **kw)
    assert run_length(full, 0) == 7
    seeds = [77]
    after_mod = oracle.run(arm, N, seeds=seeds).neutrons
    traced = oracle.run(full, N, seeds=seeds).neutrons
    passed = traced[:, 15] == 0.0
    cut = culled(full, 0, after_mod)
    assert passed.sum() > 20
    assert not (cut & passed).any(), "a neutron that passes the run was retired"
    assert cut.sum() >= 0.9 * (~passed).sum()
    scut = speed_culled(full, 0, N, seeds[0])
    assert not (scut & passed).any(), "the speed bound retired a neutron that passes"


def test_lookahead_run_detection(tmp_path):
    kw = dict(Ei=3.7, gw2=0.04, cy=0.0)
    full = instrument(tmp_path, "run.json", MOD + "," + RUN, **kw)
    assert run_length(full, 0) == 3
    assert run_length(full, 1) == 2          # from chopper 1: both choppers, no guide
    assert run_length(full, 2) == 1
    # a tapered guide, or a chopper off the axis, ends the run before it
    taper = instrument(tmp_path, "taper.json", MOD + "," + RUN, **dict(kw, gw2=0.03))
    assert run_length(taper, 0) == 0
    assert run_length(taper, 1) == 2
    off = instrument(tmp_path, "off.json", MOD + "," + RUN, **dict(kw, cy=0.01))
    assert run_length(off, 0) == 0
    assert run_length(off, 2) == 1
    # the bound is only offered where there is a run
    lib = _abi.load()
    keep = []
    _, carr, nc, barr, nb = off.descriptors(keep)
    rec = np.zeros((1, 16), np.float32)
    out = np.zeros(1, np.uint8)
    assert lib.ramp_debug_chopper_cull(ctypes.addressof(carr), nc, ctypes.addressof(barr), nb, 0,
                                       rec.ctypes.data, 1, out.ctypes.data) == _abi.E_INVALID


def test_let_like_chain_has_a_run_after_the_moderator():
    from ramp_gb300 import instruments as I
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    assert run_length(inst, 0) == 10      # guide 1 .. chopper 5, and the sample as target
    assert run_length(inst, 3) == 7       # guide 2 .. chopper 5, the sample
    slit = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs(use_slit=1))
    assert run_length(slit, 0) == 9       # the slit before the sample: no target


def test_let_like_lookahead_keeps_every_neutron_that_reaches_the_sample(tmp_path):
    """On the LET-like chain the run ends at the sample cylinder: no
    neutron that the oracle brings to the sample (its last component the
    sample or the detector) is retired by the bound from the moderator."""
    from ramp_gb300 import instruments as I
    kw = I.let_like_kwargs()
    full = m.Instrument(I.path("let_like.json"), "cpu", **kw)
    idx = {name: c["idx"] for name, c in full.components()}
    text = open(I.path("let_like.json")).read()
    body = text[text.index('"mod"'):text.index('"guide1"')].rstrip().rstrip(",")
    arm = instrument(tmp_path, "arm.json", body + "," + ARM, **kw)
    N, seeds = 2_000_000, [4321]
    after_mod = oracle.run(arm, N, seeds=seeds).neutrons
    traced = oracle.run(full, N, seeds=seeds).neutrons
    reached = np.isin(traced[:, 12].astype(int), [idx["sample"], idx["detector"]])
    cut = culled(full, 0, after_mod)
    assert reached.sum() > 50
    assert not (cut & reached).any(), "a neutron that reaches the sample was retired"
    assert cut.mean() > 0.995        # the look-ahead keeps under 0.5 %


def test_lookahead_sound_for_entries_at_guide_walls(tmp_path):
    """Guides 1 mm wide behind entrance planes exactly as wide, so that one
    neutron in about 25 enters within the position slack of a wall; choppers
    whose slit is never closed (slit_width 1.0 at radius 0.28 spans the slit
    period); a cylinder target.  Who survives depends on the entrances, the
    folding in the guides and the target only: no neutron that survives in
    the oracle is retired by the bound, and the bound does retire the ones
    that certainly miss."""
    open_chopper = ('"%s": {"position": [0.0, 0.0, %r], "geom_kernel": {"name": "GPlane", '
                    '"width": 0.6, "height": 0.6}, "scat_kernel": {"name": "SChopper", '
                    '"radius": 0.28, "freq": 300.0, "n_slits": 6, "jitter": 7e-07, '
                    '"slit_width": 1.0, "phase": 0.001}}')
    guide = ('"%s": {"position": [0.0, 0.0, %r], "geom_kernel": {"name": "GPlane", '
             '"width": 0.001, "height": 0.001}, "scat_kernel": {"name": "SGuide", "w1": 0.001, '
             '"h1": 0.001, "w2": 0.001, "h2": 0.001, "l": %r, "R0": 0.99, "Qc": 0.0219, '
             '"alpha": 3.0, "m": 3, "W": 0.003}}')
    body = ",".join([
        '"mod": {"source": true, "position": [0.0, 0.0, 0.0], "moderator_kernel": {"name": '
        '"MFlat", "mod_dim": [0.004, 0.004], "target_dim": [0.0012, 0.0012], '
        '"target_dist": 1.0, "E_min": 2.0, "E_max": 10.0}}',
        guide % ("g1", 1.0, 1.5), open_chopper % ("c1", 2.6), guide % ("g2", 2.7, 1.0),
        open_chopper % ("c2", 3.8),
        '"target": {"position": [0.0, 0.0, 4.0], "geom_kernel": {"name": "GCylinderExt", '
        '"radius": 0.0004, "height": 0.0008}, "scat_kernel": {"name": "SArm"}}'])
    full = instrument(tmp_path, "walls.json", body)
    assert run_length(full, 0) == 5
    arm = instrument(tmp_path, "arm.json", body.split(',"g1"')[0] + "," + ARM)
    N, seeds = 600_000, [99]
    after_mod = oracle.run(arm, N, seeds=seeds).neutrons
    traced = oracle.run(full, N, seeds=seeds).neutrons
    passed = traced[:, 15] == 0.0
    cut = culled(full, 0, after_mod)
    assert passed.sum() > 1000
    assert not (cut & passed).any(), "a neutron that passes was retired"
    assert cut.mean() > 0.3


def _random_run(rng):
    """IDF text of a random on-axis run behind a flat moderator: guides of
    random aperture and length and choppers of random frequency (either
    sign), slit count, slit width, radius, phase and jitter, at random
    gaps; and the moderator energy range."""
    z = float(rng.uniform(0.5, 2.0))
    mod = {"mod_dim": [float(rng.uniform(0.02, 0.12)), float(rng.uniform(0.02, 0.12))],
           "target_dim": [float(rng.uniform(0.01, 0.06)), float(rng.uniform(0.01, 0.06))],
           "target_dist": z, "E_min": float(rng.uniform(0.5, 3.0))}
    mod["E_max"] = mod["E_min"] + float(rng.uniform(0.5, 15.0))
    parts = ['"mod": {"source": true, "position": [0.0, 0.0, 0.0], "moderator_kernel": '
             '{"name": "MFlat", "mod_dim": %s, "target_dim": %s, "target_dist": %r, '
             '"E_min": %r, "E_max": %r}}' % (mod["mod_dim"], mod["target_dim"], z,
                                             mod["E_min"], mod["E_max"])]
    # every chopper phased for one design energy, as on an instrument, so
    # that a fair share of the neutrons passes the whole run
    v0 = 437.393 * np.sqrt(float(rng.uniform(mod["E_min"], mod["E_max"])))
    kinds = ["guide"] + list(rng.choice(["guide", "chopper"], size=3)) + ["chopper"]
    for j, kind in enumerate(kinds):
        if kind == "guide":
            w, h = float(rng.uniform(0.01, 0.06)), float(rng.uniform(0.01, 0.06))
            l = float(rng.uniform(0.5, 8.0))
            parts.append('"c%d": {"position": [0.0, 0.0, %r], "geom_kernel": {"name": "GPlane", '
                         '"width": %r, "height": %r}, "scat_kernel": {"name": "SGuide", "w1": %r, '
                         '"h1": %r, "w2": %r, "h2": %r, "l": %r, "R0": 0.99, "Qc": 0.0219, '
                         '"alpha": 3.0, "m": 2, "W": 0.003}}' % (j, z, w, h, w, h, w, h, l))
            z += l + float(rng.uniform(0.0, 0.5))
        else:
            parts.append('"c%d": {"position": [0.0, 0.0, %r], "geom_kernel": {"name": "GPlane", '
                         '"width": 0.6, "height": 0.6}, "scat_kernel": {"name": "SChopper", '
                         '"radius": %r, "freq": %r, "n_slits": %d, "jitter": %r, '
                         '"slit_width": %r, "phase": %r}}'
                         % (j, z, float(rng.uniform(0.1, 0.5)),
                            float(rng.choice([-1, 1]) * rng.uniform(30.0, 600.0)),
                            int(rng.integers(1, 7)), float(rng.choice([7e-7, 1e-4, 3e-3])),
                            float(rng.uniform(0.02, 0.12)),
                            float(rng.choice([-1, 1]) * z / v0)))
            z += float(rng.uniform(0.0, 0.8))
    n = len(kinds)
    if rng.uniform() < 0.5:
        # a sample cylinder after the last chopper as the run's target
        r, h = float(rng.uniform(0.01, 0.04)), float(rng.uniform(0.02, 0.1))
        parts.append('"target": {"position": [0.0, 0.0, %r], "geom_kernel": {"name": '
                     '"GCylinderExt", "radius": %r, "height": %r}, "scat_kernel": '
                     '{"name": "SArm"}}' % (z + r + float(rng.uniform(0.0, 2.0)), r, h))
        n += 1
    return ",".join(parts), n


@pytest.mark.parametrize("seed", range(24))
def test_lookahead_sound_on_random_runs(tmp_path, seed):
    """Random guide and chopper runs (a flat moderator, apertures, lengths,
    gaps, frequencies of either sign, slit counts and widths, radii, jitter
    up to 3e-3, all choppers phased for one random design energy): no
    neutron that passes the whole run in the oracle is retired by the
    bound."""
    rng = np.random.default_rng(1000 + seed)
    body, n = _random_run(rng)
    full = instrument(tmp_path, "rand.json", body)
    arm_body = body.split(',"c0"')[0] + "," + ARM
    arm = instrument(tmp_path, "arm.json", arm_body)
    assert run_length(full, 0) == n
    N = 600_000
    after_mod = oracle.run(arm, N, seeds=[seed]).neutrons
    traced = oracle.run(full, N, seeds=[seed]).neutrons
    passed = traced[:, 15] == 0.0
    cut = culled(full, 0, after_mod)
    assert passed.sum() > 50
    assert not (cut & passed).any(), "a neutron that passes the run was retired"
    scut = speed_culled(full, 0, N, seed)
    assert not (scut & passed).any(), "the speed bound retired a neutron that passes"
