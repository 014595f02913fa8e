"""The instrument chains the reference-kernel pins cover (file, kwargs),
shared by the tests and tests/golden/make_refcl_golden.py."""
import os

from ramp_gb300 import instruments as I

GOLD_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def chain(key):
    g = lambda f: os.path.join(GOLD_DIR, f)
    return {
        "small_chain": (I.path("small_chain.json"), I.small_chain_kwargs()),
        "let_like": (I.path("let_like.json"), I.let_like_kwargs()),
        "let_like_slit": (I.path("let_like.json"), I.let_like_kwargs(use_slit=1)),
        "let_like_misis": (I.path("let_like_misis.json"), I.let_like_misis_kwargs()),
        "tas_like": (I.path("tas_like.json"), I.tas_like_kwargs()),
        "powder_diffractometer": (I.path("powder_diffractometer.json"),
                                  I.powder_diffractometer_kwargs()),
        "mesh_chain": (g("mesh_chain.json"), I.mesh_imaging_kwargs(angle=0.3)),
        "rotated_chain": (g("rotated_chain.json"), I.small_chain_kwargs()),
        "nonlinear_env": (g("nonlinear_env.json"), I.small_chain_kwargs()),
        "guides_monitors": (g("guides_monitors.json"), I.small_chain_kwargs()),
    }[key]


GOLDEN_CHAINS = ["small_chain", "let_like", "let_like_slit", "let_like_misis", "tas_like",
                 "powder_diffractometer", "mesh_chain", "rotated_chain", "nonlinear_env",
                 "guides_monitors"]
