"""Golden host-side axes of the reference's SDetector1D and SDetector2D
plugins (bin counts, the 1D axis, the 2D coordinate grids): runs
mcramp/scat/detector1D.py and detector2D.py of a RAMP checkout with the
stand-ins of make_idf_golden.py and stores them in
tests/golden/detector_axes.npz.

    python tests/golden/make_detector_golden.py /path/to/RAMP
"""
import os
import sys

sys.dont_write_bytecode = True

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

BINNINGS_1D = [[-40.0, 0.25, 140.0], [0.0, 50.0, 50000.0], [50.0, 0.02, 70.0], [0.0, 0.3, 1.0],
               [-180.0, 1.0, 180.0]]
BINNINGS_2D = [([-40.0, 0.25, 140.0], [0.0, 50.0, 50000.0]),
               ([-0.03, 5.859375e-05, 0.03], [-0.03, 5.859375e-05, 0.03]),
               ([0.0, 0.3, 1.0], [2.0, 0.7, 5.0])]


def main(ref_root):
    from make_idf_golden import stubs
    from make_tas_golden import load
    stubs()
    d1 = load(ref_root, "detector1D.py", "detector1D")
    d2 = load(ref_root, "detector2D.py", "detector2D")
    out = {}
    for k, b in enumerate(BINNINGS_1D):
        det = d1.SDetector1D(binning=b, var="theta", ctx=None)
        out["axis1d_%d" % k] = np.asarray(det.axis)
    for k, (b1, b2) in enumerate(BINNINGS_2D):
        det = d2.SDetector2D(axis1_binning=b1, axis2_binning=b2, axis1_var="theta",
                             axis2_var="tof", ctx=None)
        out["X_%d" % k] = np.asarray(det.X)
        out["Y_%d" % k] = np.asarray(det.Y)
        out["n_%d" % k] = np.array([int(det.axis1_num_bins), int(det.axis2_num_bins)])
    np.savez_compressed(os.path.join(HERE, "detector_axes.npz"), **out)
    print("wrote", os.path.join(HERE, "detector_axes.npz"))


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
