"""ramp_gb300 — GB300 (sm_103a) implementation of RAMP's per-neutron
Monte-Carlo ray-tracing chain behind RAMP's instrument-definition format and
plugin classes (mcramp).  ``import ramp_gb300 as mcramp`` gives the names an
mcramp script uses: Instrument, frame_rotate, build_kernel and the plugin
classes."""
from .moderator import MFlat, MCont, MISIS
from .geom import (GPrim, GPlane, GCylinderExt, GBanana, GSphere, GSphereInt, GBox, GArm,
                   GMesh)
from .scat import (SPrim, SArm, SBeamstop, SGuide, SChopper, SIsotropic, SPowderN,
                   SDetector1D, SDetector2D, SCounter, SAttenuate, SMonochromator, SPowder1,
                   SRescal, SMCPLOut, SMCPLIn)
from .instrument import Instrument, frame_rotate, build_kernel
from .idf import Block

__version__ = "0.1.0"
