import numpy as np

from .gprim import GPrim
from .. import _abi


class GBanana(GPrim):
    """Interior of a cylinder about y, e.g. a detector bank
    (mcramp/geom/banana.py:10-87, banana.cl:3-55): hit needs t1<0<t2 and
    |y(t2)|<height/2.  The angular window is the reference's chained
    comparison ``mintheta < theta2 < maxtheta``, i.e.
    ``float(mintheta < theta2) < maxtheta`` (always true for maxtheta > 1).
    Slots: gp[0]=radius, gp[1]=height, gp[2]=mintheta, gp[3]=maxtheta."""
    kind = _abi.G_BANANA

    def __init__(self, radius=0, height=0, mintheta=0, maxtheta=0, idx=0, ctx=None):
        self.radius = np.float32(radius)
        self.height = np.float32(height)
        self.mintheta = np.float32(mintheta)
        self.maxtheta = np.float32(maxtheta)
        self.idx = idx

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.gp[0] = self.radius
        comp.gp[1] = self.height
        comp.gp[2] = self.mintheta
        comp.gp[3] = self.maxtheta

    def lines(self):
        n = 50
        lo, hi = np.radians(self.mintheta), np.radians(self.maxtheta)
        step = (hi - lo) / float(n)
        x, y, z = [], [], []
        for i in reversed(range(n)):
            y.append(self.height / 2.0); x.append(self.radius * np.sin(lo + i * step))
            z.append(self.radius * np.cos(lo + i * step))
        for i in range(n):
            y.append(-self.height / 2.0); x.append(self.radius * np.sin(lo + i * step))
            z.append(self.radius * np.cos(lo + i * step))
        x.append(x[0]); y.append(y[0]); z.append(z[0])
        return [x, y, z]
