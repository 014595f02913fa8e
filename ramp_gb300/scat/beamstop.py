import numpy as np

from .sprim import SPrim
from .. import _abi


class SBeamstop(SPrim):
    """Absorbs every neutron that reaches it (mcramp/scat/beamstop.py:8-39,
    beamstop.cl:3-32)."""
    kind = _abi.S_BEAMSTOP

    def __init__(self, idx=0, ctx=None, filename=None, **kwargs):
        self.idx = np.uint32(idx)
