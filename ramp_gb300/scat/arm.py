import numpy as np

from .sprim import SPrim
from .. import _abi


class SArm(SPrim):
    """No-op scatter (mcramp/scat/arm.py:7-37, arm.cl:3-29): resets the
    intersection and leaves the index buffer at this component."""
    kind = _abi.S_ARM

    def __init__(self, idx=0, ctx=None, **kwargs):
        self.idx = np.uint32(idx)
