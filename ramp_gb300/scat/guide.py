import numpy as np

from .sprim import SPrim
from .. import _abi


class SGuide(SPrim):
    """Tapered rectangular supermirror guide (mcramp/scat/guide.py:10-123,
    guide.cl:9-150, reflectivity include/ref.h:3-53).  Computed in FP32 (the
    reference's optional CONFIG_USE_DOUBLE build is not provided).
    Slots: sp[0..9] = w1, h1, w2, h2, l, R0, Qc, alpha, m, W;
    si[0] = max_bounces."""
    kind = _abi.S_GUIDE

    def __init__(self, w1=0, h1=0, w2=0, h2=0, l=0, R0=0, Qc=0, alpha=0, m=1, W=0, idx=0,
                 ctx=0, max_bounces=50, **kwargs):
        self.w1, self.h1, self.w2, self.h2, self.l = (np.float32(v) for v in (w1, h1, w2, h2, l))
        self.R0, self.Qc, self.alpha, self.m, self.W = (np.float32(v) for v in
                                                        (R0, Qc, alpha, m, W))
        self.idx = np.uint32(idx)
        self.max_bounces = np.uint32(max_bounces)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        for k, v in enumerate((self.w1, self.h1, self.w2, self.h2, self.l, self.R0, self.Qc,
                               self.alpha, self.m, self.W)):
            comp.sp[k] = v
        comp.si[0] = int(self.max_bounces)

    def lines(self):
        w1, h1, w2, h2, l = self.w1 / 2, self.h1 / 2, self.w2 / 2, self.h2 / 2, self.l
        x = [-w1, -w2, w2, w1, -w1, -w1, w1, w1, w2, w2, w1, -w1, -w2, w2, -w2, -w2]
        y = [h1, h2, h2, h1, h1, -h1, -h1, h1, h2, -h2, -h1, -h1, -h2, -h2, -h2, h2]
        z = [0, l, l, 0, 0, 0, 0, 0, l, l, 0, 0, l, l, l, l]
        return [x, y, z]
