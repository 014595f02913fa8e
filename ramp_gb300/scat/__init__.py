"""Scattering plugins (mcramp/scat/*)."""
from .sprim import SPrim
from .arm import SArm
from .beamstop import SBeamstop
from .guide import SGuide
from .chopper import SChopper
from .isotropic import SIsotropic, load_sqw, simps, cdf_from_pd
from .powderN import SPowderN
from .detector1D import SDetector1D
from .detector2D import SDetector2D
from .counter import SCounter
from .attenuate import SAttenuate
from .monochromator import SMonochromator
from .powder1 import SPowder1
from .rescal import SRescal
from .mcpl_io import SMCPLOut, SMCPLIn
