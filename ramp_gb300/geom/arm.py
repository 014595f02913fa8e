import numpy as np

from .gprim import GPrim
from .. import _abi


class GArm(GPrim):
    """Always-hit geometry (mcramp/geom/arm.py:7-36, arm.cl:3-22): stores
    intersection 2 = (1,1,1) so the neutron is not terminated."""
    kind = _abi.G_ARM

    def __init__(self, idx=0, ctx=None):
        self.idx = np.uint32(idx)
