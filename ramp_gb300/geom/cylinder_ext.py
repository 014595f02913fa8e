import numpy as np

from .gprim import GPrim
from .. import _abi


class GCylinderExt(GPrim):
    """Exterior of a cylinder about y (mcramp/geom/cylinder_ext.py:10-97,
    cylinder_ext.cl:3-53): hit needs 0<t1 (earlier than the stored hit),
    0<t2 and |y(t2)|<height/2.  Slots: gp[0]=radius, gp[1]=height."""
    kind = _abi.G_CYL_EXT

    def __init__(self, radius=0, height=0, idx=0, ctx=None):
        self.radius = np.float32(radius)
        self.height = np.float32(height)
        self.idx = idx

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.gp[0] = self.radius
        comp.gp[1] = self.height

    def lines(self):
        x, y, z = [], [], []
        h_2 = self.height / 2.0
        for sgn in (1.0, -1.0):
            angles = np.linspace(0, sgn * np.pi)
            for ang in angles:
                x.append(self.radius * np.sin(ang)); y.append(h_2); z.append(self.radius * np.cos(ang))
            for ang in reversed(angles):
                x.append(self.radius * np.sin(ang)); y.append(-h_2); z.append(self.radius * np.cos(ang))
            x.append(x[0]); y.append(y[0]); z.append(z[0])
        return [x, y, z]
