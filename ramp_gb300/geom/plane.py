import numpy as np

from .gprim import GPrim
from .. import _abi


class GPlane(GPrim):
    """Plane geometry (mcramp/geom/plane.py:9-77, plane.cl:3-52).

    orientation "xy" is the plane z=0, "yz" the plane x=0; a hit needs
    |x|<width/2, |y|<height/2, 0<t and v_z>0 for both orientations.
    Slots: gp[0]=width, gp[1]=height, gi[0]=orientation (0 xy, 1 yz)."""
    kind = _abi.G_PLANE

    def __init__(self, width=0, height=0, idx=0, orientation="xy", ctx=None):
        orientations = {"xy": 0, "yz": 1}
        self.orientation_str = orientation
        self.orientation = np.uint32(orientations[orientation])
        self.width = np.float32(width)
        self.height = np.float32(height)
        self.idx = np.uint32(idx)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.gp[0] = self.width
        comp.gp[1] = self.height
        comp.gi[0] = int(self.orientation)

    def lines(self):
        x = [-self.width / 2.0, self.width / 2.0, self.width / 2.0, -self.width / 2.0,
             -self.width / 2.0]
        y = [self.height / 2.0, self.height / 2.0, -self.height / 2.0, -self.height / 2.0,
             self.height / 2.0]
        z = [0.0] * 5
        return [x, y, z] if self.orientation_str == "xy" else [z, y, x]
