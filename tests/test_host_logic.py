"""Host-side logic that needs no GPU: launch settings, the autotuner's
candidate rules and cache, the CUDA-graph seed generator and the batched
instrument's checks."""
import json

import pytest

import ramp_gb300 as m
from ramp_gb300 import _abi, autotune, instruments as I
from ramp_gb300.graph import lcg_seeds


def test_tune_struct_fields_and_unknown_keys():
    t = _abi.tune_struct({"blocks_per_sm": 3, "split": 2, "walk": 1, "streams": 4})
    assert (t.blocks_per_sm, t.split, t.walk, t.streams, t.chunk) == (3, 2, 1, 4, 0)
    with pytest.raises(ValueError, match="unknown launch settings"):
        _abi.tune_struct({"blocks": 4})


def test_split_point_rule():
    """The first component reached by fewer than half of the histories,
    never one inside a non-linear block."""
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    n = 1000
    alive = [n, n, 130, 30, 16, 3, 3, 2, 2, 1, 1]
    assert autotune.split_point(inst, alive) == 2
    assert autotune.split_point(inst, [n] * 11) == 0
    assert autotune.split_point(inst, alive, threshold=0.01) == 5


def test_private_tally_candidates_only_for_small_detectors():
    assert autotune.privatizable(m.Instrument(I.path("powder_diffractometer.json"), "cpu",
                                              **I.powder_diffractometer_kwargs()))
    assert not autotune.privatizable(m.Instrument(I.path("let_like.json"), "cpu",
                                                  **I.let_like_kwargs()))   # 720 x 1000


def test_mesh_chains_get_the_walk_candidate():
    assert autotune.has_mesh(m.Instrument(I.path("mesh_imaging.json"), "cpu",
                                          **I.mesh_imaging_kwargs()))
    assert not autotune.has_mesh(m.Instrument(I.path("let_like.json"), "cpu",
                                              **I.let_like_kwargs()))


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("RAMP_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    assert autotune._load() == {}
    autotune._save({"k": {"config": {"blocks_per_sm": 4}}})
    assert json.load(open(tmp_path / "tune.json"))["k"]["config"] == {"blocks_per_sm": 4}
    assert autotune._load()["k"]["config"]["blocks_per_sm"] == 4


def test_lcg_seeds_stay_in_the_reference_range():
    seeds, state = lcg_seeds(12345, 1000)
    assert all(0 <= s <= 4096 for s in seeds)
    again, state2 = lcg_seeds(12345, 1000)
    assert seeds == again and state == state2
    first, mid = lcg_seeds(12345, 400)
    rest, end = lcg_seeds(mid, 600)
    assert first + rest == seeds and end == state


def test_batched_instrument_checks_its_variants():
    from ramp_gb300.batch import BatchedInstrument
    with pytest.raises(ValueError, match="at least one variant"):
        BatchedInstrument(I.path("let_like.json"), [], ctx="cpu")
    B = BatchedInstrument(I.path("let_like.json"),
                          [I.let_like_kwargs(Ei=3.7), I.let_like_kwargs(Ei=5.0)], ctx="cpu")
    with pytest.raises(ValueError, match="one count per variant"):
        B.execute([10])
