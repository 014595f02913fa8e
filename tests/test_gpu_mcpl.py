"""MCPL components on the GPU plain path: the dump of the surviving
neutrons (device compaction in index order, one copy to the host) against
the oracle's final records, and the load replacing the buffer."""
import os
import random

import numpy as np
import pytest

import oracle
import ramp_gb300 as m
from ramp_gb300 import _abi, instruments as I, mcpl

pytestmark = pytest.mark.gpu
GOLD_DIR = os.path.join(os.path.dirname(__file__), "golden")


def _rows(path):
    b = open(path, "rb").read()
    return np.frombuffer(b[56:], dtype=np.float32).reshape(-1, 11), b[:56]


@pytest.mark.parametrize("n", [200_000, 4099])
def test_dump_equals_oracle_survivors(cuda_lib, tmp_path, n):
    out = str(tmp_path / "dump.mcpl")
    kw = dict(I.small_chain_kwargs(), mcpl_file=repr(out), packing=repr("ramp"))
    gi = m.Instrument(os.path.join(GOLD_DIR, "mcpl_dump.json"), "cuda", **kw, no_dump=0)
    random.seed(5)
    gi.execute(n)
    ci = m.Instrument(os.path.join(GOLD_DIR, "mcpl_dump.json"), "cpu", **kw, no_dump=1)
    random.seed(5)
    r = oracle.run(ci, n)
    alive = r.neutrons[~(r.neutrons[:, 15] == 1.0)]
    assert len(alive) > 0
    want = str(tmp_path / "want.mcpl")
    mcpl.write(want, alive[:, 0:3], alive[:, 3:6], alive[:, 6:9], alive[:, 10], alive[:, 9],
               packing="ramp")
    a, ha = _rows(out)
    b, hb = _rows(want)
    assert ha == hb and a.shape == b.shape
    assert bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def test_load_replaces_the_buffer(cuda_lib, tmp_path):
    r = np.random.default_rng(8)
    k = 1000
    v = r.normal(0, 1, (k, 3))
    vel = (v / np.linalg.norm(v, axis=1)[:, None] * r.uniform(300, 3000, (k, 1))).astype(np.float32)
    src = str(tmp_path / "in.mcpl")
    mcpl.write(src, r.normal(0, 0.01, (k, 3)), vel, r.normal(0, 1, (k, 3)),
               r.uniform(0, 1e-3, k), r.uniform(0.5, 1, k), packing="mcpl")
    gi = m.Instrument(os.path.join(GOLD_DIR, "mcpl_load.json"), "cuda", mcpl_file=repr(src))
    np.random.seed(3)
    gi.execute(1500)
    recs, _ = gi.neutron_state()
    d = mcpl.read(src)
    assert np.all(recs[k:, _abi.LANE["die"]] == 1.0)
    assert np.all(recs[:k, _abi.LANE["die"]] == 0.0)
    assert np.array_equal(recs[:k, 0], (d["x"] * 1e-2).astype(np.float32))
    speed = np.linalg.norm(recs[:k, 3:6].astype(np.float64), axis=1)
    assert np.allclose(speed, 437.393377 * np.sqrt(d["ekin"] * 1e9), rtol=1e-5)
    assert np.array_equal(recs[:k, _abi.LANE["p"]], d["weight"].astype(np.float32))
    assert np.array_equal(recs[:k, _abi.LANE["tof"]], (d["time"] * 1e-3).astype(np.float32))
    mc = recs[:k, _abi.LANE["mc"]]
    assert np.all(mc >= np.arange(k)) and np.all(mc < 2 ** 30 + np.arange(k) + 1)


def test_host_components_refuse_the_fused_path(cuda_lib, tmp_path):
    kw = dict(I.small_chain_kwargs(), mcpl_file=repr(str(tmp_path / "x.mcpl")),
              packing=repr("ramp"), no_dump=0)
    gi = m.Instrument(os.path.join(GOLD_DIR, "mcpl_dump.json"), "cuda", **kw)
    with pytest.raises(ValueError, match="plain"):
        gi.execute(1000, path="fused")
