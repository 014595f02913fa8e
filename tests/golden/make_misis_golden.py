"""Golden MISIS tables from the reference's own spectrum reader.

Runs mcramp/moderator/isis_mod.py of a RAMP checkout (its MISIS class:
load_spectrum and calc_str_area) on the synthetic spectrum file written by
ramp_gb300.instruments.write_isis_spectrum, with a stand-in for pyopencl
whose buffers keep their host arrays, and stores the tables it would upload
(flux CDF, time bins, energy edges, cumulative flux at the edges), the
total, str_area and the time offset in tests/golden/misis_tables.npz.

    python tests/golden/make_misis_golden.py /path/to/RAMP
"""
import importlib.util
import os
import sys

sys.dont_write_bytecode = True   # nothing is written into the checkout
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

CASES = [  # (E_min, E_max, mod_dim, target_dim, target_dist)
    (1.1, 9.0, (0.04, 0.09), (0.04, 0.04), 1.7),
    (0.5, 50.0, (0.1, 0.1), (0.03, 0.05), 2.5),
]


def fake_pyopencl():
    cl = types.ModuleType("pyopencl")

    class mem_flags:
        READ_ONLY = 1
        COPY_HOST_PTR = 2

    class Buffer:
        def __init__(self, ctx, flags, hostbuf=None):
            self.host = np.array(hostbuf)

    class Program:
        def __init__(self, ctx, src):
            pass

        def build(self, options=None):
            return self

    cl.mem_flags, cl.Buffer, cl.Program = mem_flags, Buffer, Program
    arr = types.ModuleType("pyopencl.array")
    arr.vec = types.SimpleNamespace(float2=np.dtype([("x", np.float32), ("y", np.float32)]))
    cl.array = arr
    sys.modules["pyopencl"], sys.modules["pyopencl.array"] = cl, arr


def main(ref_root):
    from ramp_gb300.instruments import write_isis_spectrum
    fake_pyopencl()
    spec = importlib.util.spec_from_file_location(
        "ref_isis_mod", os.path.join(ref_root, "mcramp", "moderator", "isis_mod.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "spectrum.mcstas")
        write_isis_spectrum(fn)
        for k, (lo, hi, md, td, dist) in enumerate(CASES):
            m = mod.MISIS(None, spec_file=fn, mod_dim=md, target_dim=td, target_dist=dist,
                          E_min=lo, E_max=hi)
            out["c%d_flux" % k] = m.flux.host
            out["c%d_t_bins" % k] = m.time_bins.host
            out["c%d_e_bins" % k] = m.ener_bins.host
            out["c%d_e_int" % k] = m.e_int.host
            out["c%d_total" % k] = np.float32(m.total)
            out["c%d_str_area" % k] = np.float32(m.str_area)
            out["c%d_time_offset" % k] = np.float32(m.time_offset)
            out["c%d_sizes" % k] = np.array([m.num_time_bins, m.num_ener_bins], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "misis_tables.npz"), **out)
    print("wrote", os.path.join(HERE, "misis_tables.npz"), sorted(out))


def reference_root():
    """The RAMP checkout: the first argument, else $RAMP_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RAMP_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "mcramp")):
        raise SystemExit("give the RAMP checkout as the first argument or in RAMP_REFERENCE")
    return root


if __name__ == "__main__":
    main(reference_root())
