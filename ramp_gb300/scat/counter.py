import numpy as np
import torch

from .sprim import SPrim, _device
from .. import _abi


class SCounter(SPrim):
    """Scalar sum of detected weights (mcramp/scat/counter.py:11-78,
    counter.cl:18-49); marks the neutron as counted (lane se = 1)."""
    kind = _abi.S_COUNTER

    def __init__(self, idx=0, ctx=None, filename=None, **kwargs):
        self.idx = idx
        self.filename = filename
        self.counts_t = torch.zeros(2, dtype=torch.float32, device=_device(ctx))

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.tally = self.counts_t.data_ptr()
        comp.tally_err = None
        comp.tally_len = 1

    def tallies(self):
        return [self.counts_t]

    def data(self, queue=None):
        return float(self.counts_t[0].item())

    def save(self, queue=None):
        if self.filename:
            np.save(self.filename, self.data())
