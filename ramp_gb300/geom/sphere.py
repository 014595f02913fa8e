import numpy as np

from .gprim import GPrim
from .. import _abi


class GSphere(GPrim):
    """Exterior of a sphere (mcramp/geom/sphere.py:9-83, sphere.cl:3-43).
    Slots: gp[0]=radius."""
    kind = _abi.G_SPHERE

    def __init__(self, radius=0, idx=0, ctx=None):
        self.radius = np.float32(radius)
        self.idx = idx

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.gp[0] = self.radius

    def lines(self):
        a = np.linspace(0, 2 * np.pi)
        r = float(self.radius)
        x = list(np.zeros_like(a)) + list(r * np.sin(a)) + list(r * np.cos(a))
        y = list(r * np.cos(a)) + list(r * np.cos(a)) + list(np.zeros_like(a))
        z = list(r * np.sin(a)) + list(np.zeros_like(a)) + list(r * np.sin(a))
        return [x, y, z]
