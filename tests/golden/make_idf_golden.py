"""Golden instrument parses of the reference's own parser: imports the
mcramp package of a RAMP checkout with stand-ins for the modules this image
lacks (pyopencl: buffers keep their host arrays and programs do nothing;
matplotlib, mcpl, numpy-stl: empty modules; scipy.integrate.simps, removed
from SciPy: simpson), builds Instrument objects from instrument files of
this repository and records, per component in the reference's order, the
name, index, lab position and rotation, and restore flag, plus the block
structure, in tests/golden/idf_parse.json.  No bytecode is written into the
checkout.

    python tests/golden/make_idf_golden.py /path/to/RAMP
"""
import json
import os
import sys
import types

sys.dont_write_bytecode = True

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)


def cases():
    """(instrument file, keyword arguments) parsed by both parsers."""
    from ramp_gb300 import instruments as I
    G = os.path.join(ROOT, "tests", "golden")
    return [
        ("let_like.json", I.path("let_like.json"), I.let_like_kwargs(Ei=4.2, use_slit=1,
                                                                   slit_w=0.02)),
        ("powder_reference_example.json", os.path.join(G, "powder_reference_example.json"),
         dict(Ei=9.09, Mono_angle=0.4637, detector_binning=[50.0, 0.02, 70.0])),
        ("nonlinear_env.json", os.path.join(G, "nonlinear_env.json"), I.small_chain_kwargs()),
    ]


def stubs():
    from make_misis_golden import fake_pyopencl
    fake_pyopencl()
    cl = sys.modules["pyopencl"]
    for flag, v in (("READ_WRITE", 4), ("WRITE_ONLY", 8), ("ALLOC_HOST_PTR", 16)):
        setattr(cl.mem_flags, flag, v)
    cl.array.vec.float3 = np.dtype([("s0", np.float32), ("s1", np.float32),
                                    ("s2", np.float32), ("s3", np.float32)])
    cl.array.zeros = lambda queue, shape, dtype: np.zeros(shape, dtype)

    class CommandQueue:
        def __init__(self, *a, **k):
            pass
    cl.CommandQueue = CommandQueue
    cl.enqueue_copy = lambda *a, **k: None
    cl.enqueue_fill_buffer = lambda *a, **k: None
    for name in ("matplotlib", "matplotlib.pyplot", "mcpl", "stl"):
        sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["stl"].mesh = types.SimpleNamespace(Mesh=None)
    import scipy.integrate
    if not hasattr(scipy.integrate, "simps"):
        scipy.integrate.simps = scipy.integrate.simpson


class FakeCtx:
    devices = [None]


def example_cases():
    """The reference's own example instruments (examples/LET.json and
    TAS.json of the checkout, read from their directory) with the parameters
    of examples/LET_RAMP.py and TAS_RAMP.py."""
    h, mn, meV, overAA = 6.62607015e-34, 1.674929e-27, 1.602176634e-22, 1e10
    mono_d = 3.3539
    mono_q = 2 * np.pi / mono_d
    ki = 2 * np.pi / (h / np.sqrt(2 * mn * 5.0 * meV) * overAA)
    kf = ki
    rot = 1.3
    target = [float(np.sin(rot)), 0.0, float(np.cos(rot))]   # frame_rotate([0,0,1], [0,rot,0])
    let = dict(v_foc=1000.0, pha_offset=222e-6)
    return [
        ("examples/LET.json", "LET.json", let),
        # MCPL_test.json gives MFlat a toff_max keyword that MFlat does not
        # take: both parsers raise TypeError on it
        ("examples/MCPL_test.json", "MCPL_test.json", let),
        ("examples/MCPL_testback.json", "MCPL_testback.json", let),
        ("examples/TAS.json", "TAS.json",
         dict(Mono_angle=float(np.arcsin(mono_q / 2.0 / ki)), d_spacing=6.0,
              Ana_angle=float(np.arcsin(mono_q / 2.0 / kf)), monodspacing=mono_d,
              sample_target=target, sample_trot=rot)),
    ]


def component_index(c):
    """The index the parser gave a component, as its kernels keep it (the
    reference's SMCPLIn and SMCPLOut do not store theirs; their geometry
    does)."""
    for k in ("scat_kernel", "geom_kernel"):
        if hasattr(c[k], "idx"):
            return int(c[k].idx)
    return None


def parse(cases_):
    """Parses by the reference's mcramp.Instrument (stand-ins installed)."""
    import mcramp
    out = {}
    for key, fn, kw in cases_:
        try:
            inst = mcramp.Instrument(fn, FakeCtx(), None, **kw)
        except Exception as e:      # the parse fails: record how
            out[key] = {"error": type(e).__name__}
            continue
        blocks = []
        for b in inst.blocks:
            comps = []
            for name, c in b.components.items():
                comps.append({
                    "name": name,
                    "idx": component_index(c),
                    "pos": [float(c["pos"][k]) for k in ("s0", "s1", "s2")],
                    "rot": [float(c["rot"][k]) for k in ("s0", "s1", "s2")],
                    "restore": int(c["restore_neutron"]),
                })
            blocks.append({"linear": bool(b.linear), "components": comps})
        out[key] = blocks
    return out


def main(ref_root):
    stubs()
    sys.path.insert(0, ref_root)
    out = parse(cases())
    with open(os.path.join(HERE, "idf_parse.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "idf_parse.json"))


def main_examples(ref_root, out_fn):
    """Parse the checkout's examples (run from its examples directory, where
    their relative file names resolve) into out_fn."""
    stubs()
    sys.path.insert(0, ref_root)
    with open(out_fn, "w") as f:
        json.dump(parse(example_cases()), f, indent=1)


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--examples":
        main_examples(sys.argv[2], sys.argv[3])
    else:
        main(reference_root())
