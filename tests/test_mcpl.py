"""MCPL files: RAMP's writer layout byte for byte (golden bytes from the
reference's mcpl_out.py, made by tests/golden/make_mcpl_golden.py), the
standard direction packing round trip, and the reader's header handling."""
import os

import numpy as np
import pytest

from ramp_gb300 import mcpl

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "mcpl_ramp.npz"))


def test_ramp_packing_is_byte_identical_to_the_reference_writer(tmp_path):
    rec = GOLD["records"]
    alive = rec[~(rec[:, 15] == 1.0)]
    fn = str(tmp_path / "a.mcpl")
    mcpl.write(fn, alive[:, 0:3], alive[:, 3:6], alive[:, 6:9], alive[:, 10], alive[:, 9],
               packing="ramp")
    assert open(fn, "rb").read() == GOLD["mcpl_bytes"].tobytes()


@pytest.mark.parametrize("gz", [False, True])
def test_standard_packing_round_trip(tmp_path, gz):
    r = np.random.default_rng(4)
    n = 3000
    v = r.normal(0, 1, (n, 3))
    v[: n // 3, 0] *= 5
    v[n // 3: 2 * n // 3, 1] *= 5
    v[2 * n // 3:, 2] *= -5
    speed = r.uniform(200, 4000, n)
    vel = (v / np.linalg.norm(v, axis=1)[:, None] * speed[:, None]).astype(np.float32)
    pos = r.normal(0, 0.05, (n, 3)).astype(np.float32)
    pol = r.normal(0, 1, (n, 3)).astype(np.float32)
    tof = r.uniform(0, 0.02, n).astype(np.float32)
    w = r.uniform(0, 1, n).astype(np.float32)
    fn = str(tmp_path / ("b.mcpl.gz" if gz else "b.mcpl"))
    mcpl.write(fn, pos, vel, pol, tof, w, packing="mcpl")
    d = mcpl.read(fn)
    u = vel.astype(np.float64) / np.linalg.norm(vel.astype(np.float64), axis=1)[:, None]
    got = np.stack([d["ux"], d["uy"], d["uz"]], axis=1)
    assert np.abs(got - u).max() < 1e-5
    e = 5.22703725e-15 * np.linalg.norm(vel.astype(np.float64), axis=1) ** 2
    assert np.allclose(d["ekin"], e, rtol=1e-6)
    assert np.allclose(d["x"], pos[:, 0] * 100, rtol=1e-6, atol=1e-9)
    assert np.allclose(d["time"], tof * 1e3, rtol=1e-6)
    assert np.array_equal(d["weight"], w.astype(np.float64))
    assert np.all(d["pdgcode"] == 2112)


def test_reader_rejects_other_files(tmp_path):
    fn = tmp_path / "c.mcpl"
    fn.write_bytes(b"NOTMCPL" + bytes(64))
    with pytest.raises(ValueError, match="not an MCPL"):
        mcpl.read(str(fn))
    fn.write_bytes(b"MCPL003B" + bytes(64))
    with pytest.raises(ValueError, match="big-endian"):
        mcpl.read(str(fn))
