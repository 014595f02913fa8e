"""Golden host tables of the reference's SIsotropic plugin: runs
mcramp/scat/isotropic.py of a RAMP checkout (with the stand-ins of
make_idf_golden.py) on two S(q,w) files and stores q, w, the p(w) and
p(q|w) cumulative tables and the header constants in
tests/golden/sqw_host.npz.  The reference integrates with
scipy.integrate.simps, which current SciPy no longer has; the plugin is
run here with ramp_gb300.scat.isotropic.simps in its place, so the pin
covers the file parsing and the table construction around the integral
(the integral itself is the restatement's, checked against the composite
Simpson rule in tests/test_host_tables.py).

    python tests/golden/make_sqw_golden.py /path/to/RAMP
"""
import os
import sys

sys.dont_write_bytecode = True

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

SQW_FILES = ["flat_inc.sqw", "peaked_coh.sqw"]


def write_inputs():
    """The two S(q,w) files (written into tests/golden/): the flat
    vanadium-like file of the test instruments and a file with structure
    in both q and w and an uneven w grid."""
    from ramp_gb300.instruments import write_flat_sqw
    write_flat_sqw(os.path.join(HERE, "flat_inc.sqw"), nq=41)
    q = np.linspace(0.0, 6.0, 31)
    w = np.array([-2.0, -1.1, -0.5, -0.2, 0.0, 0.2, 0.5, 1.1, 2.0])
    with open(os.path.join(HERE, "peaked_coh.sqw"), "w") as f:
        f.write("# Format: Sqw data file for Isotropic_Sqw (synthetic, structured)\n")
        f.write("# V_rho 0.0412\n# sigma_abs 2.30\n# sigma_coh 11.1\n# sigma_inc 0.4\n")
        f.write("# q vector\n" + " ".join("%.6f" % v for v in q) + "\n")
        f.write("# w vector\n" + " ".join("%.6f" % v for v in w) + "\n")
        f.write("# S(q,w) matrix, one row per q\n")
        for qi in q:
            s = (1.0 + np.exp(-((qi - 2.3) / 0.3) ** 2)) * np.exp(-0.5 * (w / (0.3 + 0.2 * qi)) ** 2)
            f.write(" ".join("%.6e" % v for v in s) + "\n")


def main(ref_root):
    from make_idf_golden import stubs
    from make_tas_golden import load
    import scipy.integrate
    from ramp_gb300.scat.isotropic import simps
    stubs()
    scipy.integrate.simps = simps
    write_inputs()
    mod = load(ref_root, "isotropic.py", "isotropic")
    out = {}
    for k, fn in enumerate(SQW_FILES):
        p = mod.SIsotropic(fn_inc=os.path.join(HERE, fn), ctx=None)
        a = p.inc_args
        for j, name in enumerate(("q", "w", "pw_cdf", "pq_cdf")):
            out["%s_%d" % (name, k)] = a[j].host
        out["consts_%d" % k] = np.array([a[6], a[7], a[8]], dtype=np.float32)
    np.savez_compressed(os.path.join(HERE, "sqw_host.npz"), **out)
    print("wrote", os.path.join(HERE, "sqw_host.npz"))


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
