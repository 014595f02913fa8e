"""Golden host-side tables of the reference's SPowderN plugin: runs
mcramp/scat/powderN.py of a RAMP checkout with the pyopencl stand-in of
make_misis_golden.py (buffers keep their host arrays) and stores the line
tables (q, sigma_scat * v^2) and sigma_abs * v for a few parameter sets,
including the 40-line sample of the LET-like chain, in
tests/golden/powdern_host.npz.

    python tests/golden/make_powdern_golden.py /path/to/RAMP
"""
import os
import sys

sys.dont_write_bytecode = True   # nothing is written into the checkout

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def let_like_sample():
    """The SPowderN parameters of the LET-like chain's sample, as parsed."""
    import ramp_gb300 as m
    from ramp_gb300 import instruments as I
    inst = m.Instrument(I.path("let_like.json"), "cpu", **I.let_like_kwargs())
    sk = dict(inst.components())["sample"]["scat_kernel"]
    return dict(d_spacing=[float(x) for x in sk.d_spacing], pack=sk.pack, vc=sk.vc,
                sigma_abs=sk.sigma_abs, multiplicity=[int(x) for x in sk.multiplicity],
                DW=sk.DW, F2=[float(x) for x in sk.F2], d_phi=float(sk.d_phi))


def cases():
    return [
        let_like_sample(),
        dict(d_spacing=[3.1, 2.4, 1.9], pack=0.6, vc=60.0, sigma_abs=1.2,
             multiplicity=[6, 8, 12], DW=0.95, F2=[30.0, 12.5, 7.25], d_phi=20.0),
        dict(d_spacing=[1.1], pack=0.5, vc=121.3, sigma_abs=0.0, multiplicity=[1], DW=0.8,
             F2=[2.7], d_phi=180.0),
    ]


def main(ref_root):
    from make_misis_golden import fake_pyopencl
    from make_tas_golden import load
    fake_pyopencl()
    mod = load(ref_root, "powderN.py", "powderN")
    out = {}
    for k, c in enumerate(cases()):
        p = mod.SPowderN(ctx=None, **c)
        out["q_%d" % k] = p.q_cl.host
        out["ssv2_%d" % k] = p.sigma_scat_v2_cl.host
        out["sav_%d" % k] = np.array([p.sigma_abs_v])
    np.savez_compressed(os.path.join(HERE, "powdern_host.npz"), **out)
    print("wrote", os.path.join(HERE, "powdern_host.npz"))


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
