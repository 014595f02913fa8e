"""Golden final records of the reference's own kernels: runs a set of
instrument chains through the reference's OpenCL kernels compiled on the
host (oracle/refcl: the .cl sources of a RAMP checkout with their
reference sequencing) and stores, per chain, the final 16-lane records and
the index buffer of a seeded 1000-history chunk in
tests/golden/refcl_records.npz.

Two builds of the same kernels are recorded: "rmath" (transcendental
built-ins from ramp_gb300/csrc/rmath.h, the math library the oracle and the
CUDA kernels share: the oracle and the GPU plain path must equal these
records bit for bit) and "libm" (the C library's single-precision
functions, for configs 1 and 2 only: compared within 1e-5 relative).

    python tests/golden/make_refcl_golden.py [/path/to/RAMP]
"""
import os
import sys

sys.dont_write_bytecode = True   # nothing is written into the checkout

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

N = 1000
SEED = 2718     # the chunk seed (the reference draws it with randint(0, 4096))


def chains():
    """(key, instrument file, kwargs) of every recorded chain."""
    sys.path.insert(0, os.path.dirname(HERE))
    from tests_chains import GOLDEN_CHAINS, chain
    return [(k,) + chain(k) for k in GOLDEN_CHAINS]


LIBM_CHAINS = ("small_chain", "let_like")


def main(root):
    os.environ["RAMP_REFERENCE"] = root
    import ramp_gb300 as m
    from oracle import refcl
    out = {"n": np.int64(N), "seed": np.int64(SEED)}
    for key, fn, kw in chains():
        for math in ("rmath", "libm"):
            if math == "libm" and key not in LIBM_CHAINS:
                continue
            inst = m.Instrument(fn, "cpu", **kw)
            r = refcl.run(inst, N, math=math, seeds=[SEED])
            out["%s/%s/records" % (key, math)] = r.neutrons.copy()
            out["%s/%s/iidx" % (key, math)] = r.iidx.copy()
    np.savez_compressed(os.path.join(HERE, "refcl_records.npz"), **out)


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
