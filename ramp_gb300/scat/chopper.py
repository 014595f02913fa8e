import numpy as np

from .sprim import SPrim
from .. import _abi


class SChopper(SPrim):
    """Disk chopper (mcramp/scat/chopper.py:10-69, chopper.cl:4-59).  As in
    the reference ``freq`` is an angular frequency [rad/s] and ``phase`` is
    a time [s] (it is subtracted from the time of flight).
    Slots: sp[0..4] = slit_width, radius, freq, phase, jitter; si[0] = n_slits."""
    kind = _abi.S_CHOPPER

    def __init__(self, slit_width=0.0, radius=0.0, freq=0.0, n_slits=0, phase=0.0, jitter=0.0,
                 idx=0, ctx=0, **kwargs):
        self.slit_width = np.float32(slit_width)
        self.radius = np.float32(radius)
        self.freq = np.float32(freq)
        self.n_slits = np.uint32(n_slits)
        self.phase = np.float32(phase)
        self.jitter = np.float32(jitter)
        self.idx = np.uint32(idx)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        for k, v in enumerate((self.slit_width, self.radius, self.freq, self.phase, self.jitter)):
            comp.sp[k] = v
        comp.si[0] = int(self.n_slits)
