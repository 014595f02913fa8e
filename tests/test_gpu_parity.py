"""Parity of the CUDA paths with the CPU oracle (the reference's kernels
restated over its own record layout and sequencing).

Per-neutron final records (all 16 lanes) and the index buffer must be
bit-identical (NaN equal to NaN, +0 equal to -0): both sides run the same
FP32 operations with the same math library and one rounding per operation.
Histograms may differ only by the order of float atomic additions.  For a
bin holding H = sum(p) with E = sum(p^2), n_eff = H^2/E terms; recursive
float summation of positive terms errs by at most (n-1) u H on each side
(u = 2^-24), so per bin |gpu - cpu| <= 2 (n_eff + 1) u |H| + 1e-12 max|H|.
"""
import os
import random

import numpy as np
import pytest
import torch

import oracle
import ramp_gb300 as m
from ramp_gb300 import _abi, instruments as I
from ramp_gb300.batch import BatchedInstrument

from helpers import U32, _Host, records_equal, tallies_close  # noqa: F401
from tests_chains import GOLDEN_CHAINS, chain

pytestmark = pytest.mark.gpu

GOLD_DIR = os.path.join(os.path.dirname(__file__), "golden")
GOLD = np.load(os.path.join(GOLD_DIR, "ref_pins.npz"))
REFCL = np.load(os.path.join(GOLD_DIR, "refcl_records.npz"))


def pair(fn, kw, N, path="plain", rng="reference", chunk=None, seed=1234, tune=None):
    gi = m.Instrument(fn, "cuda", **kw)
    random.seed(seed)
    gi.execute(N, path=path, rng=rng, chunk=chunk, tune=tune)
    torch.cuda.synchronize()
    ci = m.Instrument(fn, "cpu", **kw)
    random.seed(seed)
    r = oracle.run(ci, N, chunk=chunk, rng_mode={"reference": 0, "native": 1}[rng])
    return gi, ci, r


def check_plain(fn, kw, N, **k):
    gi, ci, r = pair(fn, kw, N, **k)
    recs, iidx = gi.neutron_state()
    records_equal(recs, r.neutrons)
    assert np.array_equal(iidx, r.iidx)
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob
    assert gi.status_flags == r.flags
    return gi, ci, r


# ------------------------------------------------ the reference's kernels
@pytest.mark.parametrize("key", GOLDEN_CHAINS)
def test_plain_path_equals_reference_kernel_golden_records(cuda_lib, key):
    """The plain path against the reference's own kernels (compiled from
    its OpenCL sources on the host with the shared math library,
    tests/golden/make_refcl_golden.py): final records and index buffer of
    1000 seeded histories, bit for bit."""
    fn, kw = chain(key)
    gi = m.Instrument(fn, "cuda", **kw)
    seed = int(REFCL["seed"])
    gi.source.next_seed = lambda: seed
    gi.execute(int(REFCL["n"]), path="plain")
    torch.cuda.synchronize()
    recs, iidx = gi.neutron_state()
    records_equal(recs, REFCL["%s/rmath/records" % key])
    assert np.array_equal(iidx, REFCL["%s/rmath/iidx" % key])


# ---------------------------------------------------------------- RNG / math
def test_device_threefry_matches_reference_golden(cuda_lib):
    c0 = torch.tensor(GOLD["threefry_ctr0"].view(np.int32), device="cuda")
    tid = torch.tensor(GOLD["threefry_tid"].view(np.int32), device="cuda")
    out = torch.empty_like(c0)
    assert cuda_lib.ramp_debug_threefry(c0.data_ptr(), tid.data_ptr(), out.data_ptr(),
                                        c0.numel(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), GOLD["threefry_x"])


@pytest.mark.parametrize("fn", range(10))
def test_device_math_bit_identical_to_host(cuda_lib, fn):
    r = np.random.default_rng(fn)
    a = np.concatenate([r.uniform(-20, 20, 50000), r.standard_normal(50000),
                        np.exp(r.uniform(-30, 30, 50000)), r.uniform(-1, 1, 50000),
                        [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan]]).astype(np.float32)
    if fn == 9:
        a = np.abs(r.uniform(0, 0.2, 200007)).astype(np.float32)
    b = np.roll(a, 7)
    host = oracle.math(fn, a, b)
    da, db = torch.tensor(a, device="cuda"), torch.tensor(b, device="cuda")
    out = torch.empty_like(da)
    assert cuda_lib.ramp_debug_math(fn, da.data_ptr(), db.data_ptr(), out.data_ptr(),
                                    da.numel(), None) == 0
    torch.cuda.synchronize()
    dev = out.cpu().numpy()
    same = (dev.view(np.uint32) == host.view(np.uint32)) | (np.isnan(dev) & np.isnan(host))
    assert same.all(), "fn %d: %d differ" % (fn, (~same).sum())


# ---------------------------------------------------------------- plain path
def test_small_chain_plain_matches_oracle(cuda_lib):
    check_plain(I.path("small_chain.json"), I.small_chain_kwargs(), 300_000)


def test_let_like_plain_matches_oracle(cuda_lib):
    check_plain(I.path("let_like.json"), I.let_like_kwargs(), 1_000_000)


def test_let_like_with_slit_and_other_ei(cuda_lib):
    check_plain(I.path("let_like.json"), I.let_like_kwargs(Ei=12.0, use_slit=1, slit_w=0.02),
                400_000)


def test_mesh_imaging_bvh_matches_brute_force_oracle(cuda_lib):
    check_plain(I.path("mesh_imaging.json"), I.mesh_imaging_kwargs(angle=0.37), 20_000)


@pytest.mark.parametrize("name", ["nonlinear_env.json", "rotated_chain.json",
                                  "guides_monitors.json"])
def test_feature_chains_match_oracle(cuda_lib, name):
    check_plain(os.path.join(GOLD_DIR, name), I.small_chain_kwargs(), 200_000)


@pytest.mark.parametrize("N", [1, 37, 1000, 4099])
def test_ragged_sizes(cuda_lib, N):
    check_plain(I.path("small_chain.json"), I.small_chain_kwargs(), N)


def test_multi_chunk_reference_keying(cuda_lib):
    """Three chunks (the last one short): counters carry over between chunks
    (flat_mod.cl:19) and weights are 1/N_chunk."""
    check_plain(I.path("small_chain.json"), I.small_chain_kwargs(), 250_001, chunk=100_000)


def test_native_keying_matches_oracle(cuda_lib):
    check_plain(I.path("let_like.json"), I.let_like_kwargs(), 500_000, rng="native")


def test_misis_chain_plain_matches_oracle(cuda_lib):
    """The tabulated ISIS moderator: bisection on the device, the
    reference's linear scan in the oracle; records bit-identical."""
    check_plain(I.path("let_like_misis.json"), I.let_like_misis_kwargs(), 300_000)


def test_misis_chain_fused_and_native(cuda_lib):
    gi, ci, r = pair(I.path("let_like_misis.json"), I.let_like_misis_kwargs(), 400_000,
                     path="fused")
    tallies_close(gi, ci)
    check_plain(I.path("let_like_misis.json"), I.let_like_misis_kwargs(), 100_000, rng="native")


def test_misis_rejects_decreasing_tables(cuda_lib):
    inst = m.Instrument(I.path("let_like_misis.json"), "cuda", **I.let_like_misis_kwargs())
    inst.source.spectrum = dict(inst.source.spectrum)
    flux = inst.source.spectrum["flux"].copy()
    flux[5] = flux[4] - 1.0
    inst.source.spectrum["flux"] = flux
    with pytest.raises(RuntimeError, match="decreases"):
        inst.execute(1000)


@pytest.mark.parametrize("rng", ["reference", "native"])
def test_powder_diffractometer_plain_matches_oracle(cuda_lib, rng):
    """Curved mosaic monochromator (slab tilts, Bragg orders, mosaic
    quadrature, Box-Muller draw) and a one-line powder: records
    bit-identical."""
    check_plain(I.path("powder_diffractometer.json"), I.powder_diffractometer_kwargs(),
                300_000, rng=rng)


def test_powder_diffractometer_fused_matches_oracle(cuda_lib):
    gi, ci, r = pair(I.path("powder_diffractometer.json"), I.powder_diffractometer_kwargs(),
                     500_000, path="fused")
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob


def test_tas_like_plain_matches_oracle_with_events(cuda_lib):
    """Monochromator, SRescal with its per-index event list, analyser and
    counter: records and the kept events bit-identical."""
    gi, ci, r = check_plain(I.path("tas_like.json"), I.tas_like_kwargs(), 300_000)
    g = dict(gi.components())["Sample"]["scat_kernel"].data()
    c = dict(ci.components())["Sample"]["scat_kernel"].data()
    assert len(g[0]) == len(c[0]) > 0
    for a, b in zip(g, c):
        assert np.array_equal(a, b)


def test_rescal_plan_refuses_whole_chain_launches(cuda_lib):
    inst = m.Instrument(I.path("tas_like.json"), "cuda", **I.tas_like_kwargs())
    inst.execute(1000)
    lib = inst._lib()
    rngd = _abi.RampRng()
    rc = lib.ramp_trace_fused(inst.plan(), 1000, 1000, 1, _abi.ctypes.byref(rngd), None, None,
                              None, None)
    assert rc == _abi.E_UNSUPPORTED


# ---------------------------------------------------------------- fused path
@pytest.mark.parametrize("fn,kw,N", [
    ("small_chain.json", "small", 300_000),
    ("let_like.json", "let", 1_000_000),
    ("mesh_imaging.json", "mesh", 20_000)])
def test_fused_matches_oracle(cuda_lib, fn, kw, N):
    kws = {"small": I.small_chain_kwargs(), "let": I.let_like_kwargs(),
           "mesh": I.mesh_imaging_kwargs(0.37)}[kw]
    gi, ci, r = pair(I.path(fn), kws, N, path="fused")
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob


@pytest.mark.parametrize("name", ["nonlinear_env.json", "rotated_chain.json",
                                  "guides_monitors.json"])
def test_fused_feature_chains(cuda_lib, name):
    gi, ci, r = pair(os.path.join(GOLD_DIR, name), I.small_chain_kwargs(), 200_000,
                     path="fused")
    tallies_close(gi, ci)


def test_fused_multi_chunk_carry(cuda_lib):
    gi, ci, r = pair(I.path("small_chain.json"), I.small_chain_kwargs(), 250_001, path="fused",
                     chunk=100_000)
    tallies_close(gi, ci)


def test_fused_native_keying(cuda_lib):
    gi, ci, r = pair(I.path("let_like.json"), I.let_like_kwargs(), 500_000, path="fused",
                     rng="native")
    tallies_close(gi, ci)


def test_fused_equals_plain_at_1e7(cuda_lib):
    """Size-independent property at full size: the fused and plain paths
    trace the same histories, so their tallies agree to reordering error."""
    kw = I.let_like_kwargs()
    a = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    b = m.Instrument(I.path("let_like.json"), "cuda", **kw)
    random.seed(7)
    a.execute(10_000_000, path="plain")
    random.seed(7)
    b.execute(10_000_000, path="fused")
    tallies_close(b, _Host(a))


# ---------------------------------------------------------------- batching
@pytest.mark.parametrize("tune", [None, {"streams": 1, "blocks_per_sm": 3},
                                  {"streams": 2, "blocks_per_sm": 4}, {"streams": 16}])
def test_batched_variants_match_single_runs(cuda_lib, tune):
    """Variants with different Ei, slit width and neutron count, traced as
    one launch with a grid row per variant (default, streams 1) or as
    per-variant launches on 2 or 16 streams; each equals its own oracle
    run with the same seed and keying."""
    variants = [I.let_like_kwargs(Ei=3.7, use_slit=1, slit_w=0.03),
                I.let_like_kwargs(Ei=8.0, use_slit=1, slit_w=0.015),
                I.let_like_kwargs(Ei=2.5, use_slit=1, slit_w=0.04)]
    counts = [300_000, 123_457, 200_003]
    for mode, rng in ((0, "reference"), (1, "native")):
        B = BatchedInstrument(I.path("let_like.json"), variants, ctx="cuda")
        B.execute(counts, rng=rng, seeds=[11, 2222, 4000], tune=tune)
        torch.cuda.synchronize()
        for v, (kw, n, seed) in enumerate(zip(variants, counts, [11, 2222, 4000])):
            ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
            oracle.run(ci, n, rng_mode=mode, variant=v, seeds=[seed])
            tallies_close(B.instruments[v], ci)


# ------------------------------------------------- survivor compaction
@pytest.mark.parametrize("fn,kw,N,split,rng", [
    ("small_chain.json", "small", 300_000, 1, "reference"),
    ("small_chain.json", "small", 300_000, 2, "native"),
    ("let_like.json", "let", 1_000_000, 2, "reference"),
    ("let_like.json", "let", 1_000_000, 5, "native"),
    ("mesh_imaging.json", "mesh", 20_000, 1, "reference"),
    ("let_like_misis.json", "misis", 400_000, 2, "reference"),
    ("powder_diffractometer.json", "powder", 500_000, 3, "native")])
def test_fused_split_matches_oracle(cuda_lib, fn, kw, N, split, rng):
    """Compacting survivors into full warps changes only the order in
    which neutrons are traced (also with the extended kinds: MISIS source,
    SMonochromator in stage A, SPowder1 in stage B)."""
    kws = {"small": I.small_chain_kwargs(), "let": I.let_like_kwargs(),
           "mesh": I.mesh_imaging_kwargs(0.37), "misis": I.let_like_misis_kwargs(),
           "powder": I.powder_diffractometer_kwargs()}[kw]
    gi, ci, r = pair(I.path(fn), kws, N, path="fused", rng=rng, tune={"split": split})
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob


@pytest.mark.parametrize("tune,chunk,rng", [({"walk": 1}, None, "reference"),
                                             ({"walk": 1, "blocks_per_sm": 3}, None, "native"),
                                             ({"walk": 1}, 7_000, "reference")])
def test_fused_mesh_walk_matches_oracle(cuda_lib, tune, chunk, rng):
    """Stage B walking the mesh one node per pass on each lane, lanes taking
    the next waiting ray when their walk is over (the mesh is component 0,
    so stage A is the moderator alone); with carry buffers across chunks."""
    gi, ci, r = pair(I.path("mesh_imaging.json"), I.mesh_imaging_kwargs(0.37), 20_000,
                     path="fused", rng=rng, chunk=chunk, tune=tune)
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob


@pytest.mark.parametrize("tune", [{"walk": 1}, {"walk": 1, "streams": 4}])
def test_batched_mesh_walk_matches_single_runs(cuda_lib, tune):
    """Three views of the mesh in one call (grid rows or streams), walked
    per lane; each equals its own oracle run."""
    angles, counts, seeds = [0.0, 0.7, 2.1], [9_000, 5_001, 7_777], [3, 4, 5]
    variants = [I.mesh_imaging_kwargs(angle=t) for t in angles]
    B = BatchedInstrument(I.path("mesh_imaging.json"), variants, ctx="cuda")
    B.execute(counts, rng="native", seeds=seeds, tune=tune)
    torch.cuda.synchronize()
    for v, (kw, n, seed) in enumerate(zip(variants, counts, seeds)):
        ci = m.Instrument(I.path("mesh_imaging.json"), "cpu", **kw)
        oracle.run(ci, n, rng_mode=1, variant=v, seeds=[seed])
        tallies_close(B.instruments[v], ci)


@pytest.mark.parametrize("split", [1, 4])
def test_fused_split_at_nonlinear_block_boundaries(cuda_lib, split):
    gi, ci, r = pair(os.path.join(GOLD_DIR, "nonlinear_env.json"), I.small_chain_kwargs(),
                     200_000, path="fused", tune={"split": split})
    tallies_close(gi, ci)


def test_fused_split_inside_nonlinear_block_is_refused(cuda_lib):
    gi = m.Instrument(os.path.join(GOLD_DIR, "nonlinear_env.json"), "cuda",
                      **I.small_chain_kwargs())
    with pytest.raises(RuntimeError, match="non-linear block"):
        gi.execute(1000, path="fused", tune={"split": 2})
    with pytest.raises(RuntimeError, match="components"):
        gi.execute(1000, path="fused", tune={"split": 99})


def test_fused_split_with_multi_chunk_carry(cuda_lib):
    """Carry buffers are written when each neutron finishes, parked or not."""
    gi, ci, r = pair(I.path("let_like.json"), I.let_like_kwargs(), 250_001, path="fused",
                     chunk=100_000, tune={"split": 2})
    tallies_close(gi, ci)


@pytest.mark.parametrize("fn,kw,N,tune", [
    ("powder_diffractometer.json", "powder", 500_000, {"privatize": 1}),
    ("guides_monitors.json", "small", 300_000, {"privatize": 1, "blocks_per_sm": 3}),
    ("let_like.json", "let", 1_000_000, {"block": 128, "blocks_per_sm": 8, "split": 2}),
    ("let_like.json", "let", 600_001, {"block": 128, "blocks_per_sm": 6})])
def test_fused_private_tallies_and_small_ctas_match_oracle(cuda_lib, fn, kw, N, tune):
    """Detectors whose histograms fit in shared memory accumulated per CTA
    and merged as the CTA ends (the powder diffractometer's 1600-bin 2theta
    histogram, the monitors of the guide chain), and 128-thread CTAs: only
    the order of tally additions changes."""
    kws = {"small": I.small_chain_kwargs(), "let": I.let_like_kwargs(),
           "powder": I.powder_diffractometer_kwargs()}[kw]
    path = os.path.join(GOLD_DIR, fn) if fn == "guides_monitors.json" else I.path(fn)
    gi, ci, r = pair(path, kws, N, path="fused", tune=tune)
    tallies_close(gi, ci)
    assert gi.oob_drops == r.oob


@pytest.mark.parametrize("tune", [{"split": 2}, {"split": 2, "streams": 4}])
def test_batched_split_matches_single_runs(cuda_lib, tune):
    """Split batched launches: per-variant launches, or one launch with a
    grid row per variant; either way each variant has its own survivor
    range and stage-B counter."""
    variants = [I.let_like_kwargs(Ei=3.7), I.let_like_kwargs(Ei=8.0), I.let_like_kwargs(Ei=2.5)]
    counts = [300_000, 123_457, 200_003]
    B = BatchedInstrument(I.path("let_like.json"), variants, ctx="cuda")
    B.execute(counts, rng="native", seeds=[11, 2222, 4000], tune=tune)
    torch.cuda.synchronize()
    for v, (kw, n, seed) in enumerate(zip(variants, counts, [11, 2222, 4000])):
        ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
        oracle.run(ci, n, rng_mode=1, variant=v, seeds=[seed])
        tallies_close(B.instruments[v], ci)


@pytest.mark.parametrize("tune", [None, {"split": 2}, {"streams": 4}])
def test_batched_empty_and_ragged_variants(cuda_lib, tune):
    """Variants of 0, 1, 37 and 200,003 histories in one call: the empty
    one tallies nothing, the others equal their own oracle runs."""
    variants = [I.let_like_kwargs(Ei=e) for e in (3.7, 5.0, 2.5, 3.7)]
    counts, seeds = [0, 1, 37, 200_003], [9, 10, 11, 12]
    B = BatchedInstrument(I.path("let_like.json"), variants, ctx="cuda")
    B.execute(counts, rng="native", seeds=seeds, tune=tune)
    torch.cuda.synchronize()
    assert all(float(t.abs().sum()) == 0.0 for t in B.instruments[0].tallies())
    for v in range(1, 4):
        ci = m.Instrument(I.path("let_like.json"), "cpu", **variants[v])
        oracle.run(ci, counts[v], rng_mode=1, variant=v, seeds=[seeds[v]])
        tallies_close(B.instruments[v], ci)


@pytest.mark.parametrize("tune", [{"split": 2}, {"split": 2, "streams": 4}])
def test_batched_misis_split_matches_single_runs(cuda_lib, tune):
    """MISIS variants: the one-launch layout runs the extended kinds
    whole; per-variant launches split them."""
    variants = [I.let_like_misis_kwargs(Ei=3.7), I.let_like_misis_kwargs(Ei=6.0)]
    counts, seeds = [250_000, 99_999], [5, 3001]
    B = BatchedInstrument(I.path("let_like_misis.json"), variants, ctx="cuda")
    B.execute(counts, rng="native", seeds=seeds, tune=tune)
    torch.cuda.synchronize()
    for v, (kw, n, seed) in enumerate(zip(variants, counts, seeds)):
        ci = m.Instrument(I.path("let_like_misis.json"), "cpu", **kw)
        oracle.run(ci, n, rng_mode=1, variant=v, seeds=[seed])
        tallies_close(B.instruments[v], ci)


def test_autotune_survival_and_split_point(cuda_lib, tmp_path, monkeypatch):
    from ramp_gb300 import autotune
    monkeypatch.setenv("RAMP_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    inst = m.Instrument(I.path("let_like.json"), "cuda", **I.let_like_kwargs())
    alive = autotune.survival(inst, 200_000)
    assert alive[0] == 200_000 and all(a >= b for a, b in zip(alive, alive[1:]))
    # the first chopper passes a few per cent: compaction goes before the second
    assert autotune.split_point(inst, alive) == 2
    before = [t.clone() for t in inst.tallies()]
    cfg = autotune.tune(inst, n_probe=200_000)
    assert set(cfg) <= set(("block", "blocks_per_sm", "chunk", "split", "privatize", "cull"))
    assert autotune.chopper_run_start(inst) == 0
    for t, b in zip(inst.tallies(), before):
        assert torch.equal(t, b)


# ------------------------------------------------ statistical agreement
def _chi2_two_sample(h1, e1, h2, e2, min_count=0.0):
    """Two-sample chi-square of weighted histograms (sum p, sum p^2 per bin)
    over the bins whose pooled effective count (h1 + h2)^2 / (e1 + e2)
    reaches min_count (a cut symmetric in the two samples)."""
    from scipy.stats import chi2
    v = e1 + e2
    n_eff = np.where(v > 0, (h1 + h2) ** 2 / np.where(v > 0, v, 1.0), 0.0)
    use = (v > 0) & (n_eff >= min_count)
    stat = float((((h1 - h2) ** 2)[use] / v[use]).sum())
    dof = int(use.sum())
    return stat, dof, float(chi2.sf(stat, dof))


@pytest.mark.parametrize("fn,kw,N,shape,min_count,tune", [
    # 500 x 500 (2theta x TOF) detector rebinned to 50 x 50: both axes kept
    ("small_chain.json", "small", 10_000_000, (50, 10, 50, 10), 5.0, None),
    # the LET-like detector at its full 50-us TOF resolution (the axis the
    # five choppers shape) and 2.5-degree angle bins
    ("let_like.json", "let", 200_000_000, (72, 10, 1000, 1), 3.0, None),
    # the same with the chopper look-ahead (one chunk per call: it stands
    # aside when RNG counters are carried between chunks)
    ("let_like.json", "let", 200_000_000, (72, 10, 1000, 1), 3.0, {"split": 0, "cull": 1})])
def test_fused_agrees_with_oracle_on_independent_streams(cuda_lib, fn, kw, N, shape, min_count,
                                                         tune):
    """Different chunk seeds (independent random streams): the fused GPU
    histogram and the oracle's pass a two-sample chi-square test, p > 0.01,
    on a two-dimensional (angle x time-of-flight) rebinning of the
    detector, over the bins with a pooled effective count >= min_count."""
    kws = {"small": I.small_chain_kwargs(), "let": I.let_like_kwargs()}[kw]
    gi = m.Instrument(I.path(fn), "cuda", **kws)
    chunk = 10_000_000             # the same chunk weights 1/N_chunk on both sides
    random.seed(101)
    if tune is None:
        gi.execute(N, path="fused", chunk=chunk)
    else:
        for _ in range(N // chunk):
            gi.execute(chunk, path="fused", tune=tune)
    torch.cuda.synchronize()
    ci = m.Instrument(I.path(fn), "cpu", **kws)
    random.seed(202)
    oracle.run(ci, N, chunk=chunk)
    g = [t.double().cpu().numpy() for t in gi.tallies()[-2:]]
    c = [t.double().numpy() for t in ci.tallies()[-2:]]
    a, b, d, e = shape
    rb = lambda x: x.reshape(a, b, d, e).sum(axis=(1, 3))
    stat, dof, p = _chi2_two_sample(rb(g[0]), rb(g[1]), rb(c[0]), rb(c[1]), min_count)
    assert dof > 10 and p > 0.01, (stat, dof, p)
    # the tested bins span several time-of-flight bins, not one per angle
    used = np.argwhere(rb(c[0]) > 0)
    assert len(np.unique(used[:, 1])) > 3


# ---------------------------------------------------------------- shards
@pytest.mark.parametrize("path", ["plain", "fused"])
def test_shards_sum_to_single_run(cuda_lib, path):
    """Two shards traced one after the other on this GPU (no collective):
    their tallies sum to the oracle's single run, including a short last
    chunk whose slice is clipped for the higher rank."""
    kw = I.let_like_kwargs()
    N, chunk = 250_001, 100_000
    parts = []
    for rank in range(2):
        gi = m.Instrument(I.path("let_like.json"), "cuda", **kw)
        random.seed(77)
        gi.execute(N, path=path, chunk=chunk, shard=(rank, 2))
        parts.append([t.double().cpu() for t in gi.tallies()])
    torch.cuda.synchronize()

    class Summed:
        def tallies(self):
            return [(a + b).float() for a, b in zip(*parts)]

    ci = m.Instrument(I.path("let_like.json"), "cpu", **kw)
    random.seed(77)
    oracle.run(ci, N, chunk=chunk)
    tallies_close(Summed(), ci)


# ---------------------------------------------------------------- status
def test_guide_bounce_cap_and_oob_counts(cuda_lib):
    gi, ci, r = check_plain(os.path.join(GOLD_DIR, "guides_monitors.json"),
                            I.small_chain_kwargs(), 100_000)
    assert r.oob > 0 and gi.oob_drops == r.oob
