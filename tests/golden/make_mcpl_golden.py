"""Golden bytes of RAMP's MCPL writer: runs write_hdr and write_particle of
mcpl_out.py (a RAMP checkout, pyopencl replaced by a stand-in) on seeded
synthetic neutron records and stores records and file bytes in
tests/golden/mcpl_ramp.npz.

    python tests/golden/make_mcpl_golden.py /path/to/RAMP
"""
import importlib.util
import io
import os
import sys

sys.dont_write_bytecode = True   # nothing is written into the checkout

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def records(n=257, seed=9):
    r = np.random.default_rng(seed)
    rec = np.zeros((n, 16), dtype=np.float32)
    rec[:, 0:3] = r.normal(0, 0.02, (n, 3))
    v = r.normal(0, 1, (n, 3))
    v[: n // 3, 2] = np.abs(v[: n // 3, 2]) * 5          # mostly forward
    v[n // 3: n // 2, 0] *= 4                           # x-dominant
    v[n // 2: 2 * n // 3, 1] *= 4                       # y-dominant
    rec[:, 3:6] = v / np.linalg.norm(v, axis=1)[:, None] * r.uniform(300, 3000, (n, 1))
    rec[:, 6:9] = r.normal(0, 1, (n, 3))
    rec[:, 9] = r.uniform(0, 1e-3, n)
    rec[:, 10] = r.uniform(0, 0.05, n)
    rec[:, 15] = (r.uniform(0, 1, n) < 0.2).astype(np.float32)   # some dead
    rec[:5, 3:6] = [[1, 2, 3], [-1, -2, -3], [3, 2, 1], [0, 0, 0], [2, 2, 1]]
    return rec


def main(ref_root):
    from make_misis_golden import fake_pyopencl
    fake_pyopencl()
    spec = importlib.util.spec_from_file_location(
        "ref_mcpl_out", os.path.join(ref_root, "mcramp", "scat", "mcpl_out.py"))
    sys.modules["ref_sprim_pkg"] = None
    src = open(os.path.join(ref_root, "mcramp", "scat", "mcpl_out.py")).read()
    src = src.replace("from .sprim import SPrim", "SPrim = object")
    mod = type(sys)("ref_mcpl_out")
    exec(compile(src, "mcpl_out.py", "exec"), mod.__dict__)
    rec = records()
    buf = io.BytesIO()
    alive = [row for row in rec if not row[15] == 1.0]
    for row in alive:
        mod.write_particle(buf, row)
    body = buf.getvalue()
    hdr = io.BytesIO()
    mod.write_hdr(hdr, len(alive))
    np.savez_compressed(os.path.join(HERE, "mcpl_ramp.npz"), records=rec,
                        mcpl_bytes=np.frombuffer(hdr.getvalue() + body, dtype=np.uint8))
    print("wrote", os.path.join(HERE, "mcpl_ramp.npz"), len(alive), "particles")


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
