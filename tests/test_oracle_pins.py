"""The oracle's RNG and reflectivity against the reference's own code
(golden fixtures made by tests/golden/make_golden.py from the reference's
rand.h / Random123 / ref.h; and live when the reference checkout exists)."""
import os

import numpy as np
import pytest

import oracle

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_pins.npz"))


def test_threefry_kat_matches_reference():
    x = oracle.threefry(GOLD["threefry_ctr0"], GOLD["threefry_tid"])
    assert np.array_equal(x, GOLD["threefry_x"])
    # the known answer quoted for (tid 0, counter 0)
    assert GOLD["threefry_x"][0] == 0x5cab7cde


def test_rand_sequences_match_reference():
    L = oracle.lib()
    for t, sb0, us, sbs in zip(GOLD["rand_tid"], GOLD["rand_sb0"], GOLD["rand_u"],
                               GOLD["rand_sb"]):
        rec = np.zeros(16, np.float32)
        rec[11] = sb0
        for u, sb in zip(us, sbs):
            got = L.oracle_rand(rec.ctypes.data, int(t), 0, 0, 0)
            assert np.float32(got) == u
            assert rec[11] == sb


def test_first_draw_known_answer():
    rec = np.zeros(16, np.float32)
    assert np.float32(oracle.lib().oracle_rand(rec.ctypes.data, 0, 0, 0, 0)) == np.float32(
        0.723983407)
    assert rec[11] == 1.0


def test_reflectivity_matches_reference():
    """FP32 restatement vs the reference compiled as C (which evaluates its
    unsuffixed constants in double): equal to 2.5e-7 absolute, i.e. within
    about two float ulps of R0, everywhere; within 1e-5 relative where
    R > 1e-2."""
    L = oracle.lib()
    for prm, Rref in zip(GOLD["refl_params"], GOLD["refl_R"]):
        got = np.array([L.oracle_reflectivity(float(q), *[float(v) for v in prm])
                        for q in GOLD["refl_q"]], np.float32)
        assert np.max(np.abs(got - Rref)) <= 2.5e-7
        big = Rref > 1e-2
        if big.any():
            assert np.max(np.abs(got[big] - Rref[big]) / Rref[big]) < 1e-5
        # the cut-offs agree exactly
        assert np.array_equal(got == 0, Rref == 0) or np.max(np.abs(got - Rref)) < 2.5e-7


def test_live_reference_pins_when_available():
    P = oracle.pins()
    if P is None:
        pytest.skip("reference checkout not available")
    rng = np.random.default_rng(3)
    c0 = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
    tid = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
    ref = np.zeros_like(c0)
    P.ref_pin_threefry(c0.ctypes.data, tid.ctypes.data, ref.ctypes.data, c0.size)
    assert np.array_equal(oracle.threefry(c0, tid), ref)


# ------------------------------------------------ the reference's kernels
REFCL = np.load(os.path.join(os.path.dirname(__file__), "golden", "refcl_records.npz"))
REFCL_CHAINS = sorted({k.split("/")[0] for k in REFCL.files if "/" in k})


@pytest.mark.parametrize("key", REFCL_CHAINS)
def test_oracle_equals_reference_kernel_golden_records(key):
    """Final records of 1000 seeded histories of each chain, as the
    reference's own kernels compute them with the shared math library
    (tests/golden/make_refcl_golden.py): the oracle gives the same bits."""
    import ramp_gb300 as m
    from helpers import records_equal
    from tests_chains import chain
    fn, kw = chain(key)
    r = oracle.run(m.Instrument(fn, "cpu", **kw), int(REFCL["n"]), seeds=[int(REFCL["seed"])])
    records_equal(r.neutrons, REFCL["%s/rmath/records" % key])
    assert np.array_equal(r.iidx, REFCL["%s/rmath/iidx" % key])


@pytest.mark.parametrize("key", ["small_chain", "let_like"])
def test_oracle_within_1e5_of_reference_kernels_with_the_c_math_library(key):
    """The same chains through the reference kernels built with the C
    library's math: same branches, vectors and times within 1e-5."""
    import ramp_gb300 as m
    from tests_chains import chain
    fn, kw = chain(key)
    r = oracle.run(m.Instrument(fn, "cpu", **kw), int(REFCL["n"]), seeds=[int(REFCL["seed"])])
    x = r.neutrons.astype(np.float64)
    y = REFCL["%s/libm/records" % key].astype(np.float64)
    assert np.array_equal(r.iidx, REFCL["%s/libm/iidx" % key])
    assert np.array_equal(x[:, [11, 12, 15]], y[:, [11, 12, 15]])
    for lo in (0, 3, 6):
        d = np.linalg.norm(x[:, lo:lo + 3] - y[:, lo:lo + 3], axis=1)
        assert (d <= 1e-5 * np.linalg.norm(x[:, lo:lo + 3], axis=1)).all()
    assert (np.abs(x[:, 10] - y[:, 10]) <= 1e-5 * np.abs(x[:, 10])).all()
