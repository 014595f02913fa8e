"""Golden host-side values of the reference's SMonochromator and SPowder1
plugins: runs mcramp/scat/monochromator.py and powder1.py of a RAMP
checkout with a stand-in for pyopencl (buffers keep their host arrays,
programs do nothing) and stores the monochromator's quadrature tables and
the powder line constants for a few parameter sets in
tests/golden/tas_host.npz.

    python tests/golden/make_tas_golden.py /path/to/RAMP
"""
import importlib.util
import os
import sys

sys.dont_write_bytecode = True   # nothing is written into the checkout
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

POWDER1_CASES = [  # d_spacing, pack, vc, sigma_abs, multiplicity, DW, F2, d_phi
    (2.5, 0.6, 60.0, 1.2, 6, 0.95, 30.0, 20.0),
    (3.0, 1.0, 75.0, 0.0, 1, 1.0, 500.0, 30.0),
    (1.1, 0.5, 121.3, 5.08, 12, 0.8, 2.7, 0.0),
]


def load(ref_root, rel, name):
    pkg = types.ModuleType("refscat")
    pkg.__path__ = [os.path.join(ref_root, "mcramp", "scat")]
    sys.modules["refscat"] = pkg
    spec = importlib.util.spec_from_file_location(
        "refscat." + name, os.path.join(ref_root, "mcramp", "scat", rel))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["refscat." + name] = mod
    spec.loader.exec_module(mod)
    return mod


def main(ref_root):
    from make_misis_golden import fake_pyopencl
    fake_pyopencl()
    mono = load(ref_root, "monochromator.py", "monochromator")
    pw1 = load(ref_root, "powder1.py", "powder1")
    out = {}
    m = mono.SMonochromator(slab_width=0.02, slab_height=0.02, d_spacing=3.355, ctx=None)
    out["gauss_x"] = m.gaussX_opencl.host
    out["gauss_w"] = m.gaussW_opencl.host
    rows = []
    for c in POWDER1_CASES:
        p = pw1.SPowder1(*c, ctx=None)
        rows.append([p.sigma_scat_v2, p.sigma_abs_v, p.q, p.d_phi])
    out["powder1"] = np.array(rows, dtype=np.float32)
    out["powder1_cases"] = np.array(POWDER1_CASES, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "tas_host.npz"), **out)
    print("wrote", os.path.join(HERE, "tas_host.npz"))


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
