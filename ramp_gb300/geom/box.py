import numpy as np

from .gprim import GPrim
from .. import _abi


class GBox(GPrim):
    """Axis-aligned box, slab test (mcramp/geom/box.py:9-81, box.cl:3-53).
    As in the reference a hit overwrites the stored intersection without an
    earliest-hit comparison.  Slots: gp[0..2]=width, height, depth."""
    kind = _abi.G_BOX

    def __init__(self, width=0, height=0, depth=0, idx=0, ctx=None):
        self.width = np.float32(width)
        self.height = np.float32(height)
        self.depth = np.float32(depth)
        self.idx = idx

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.gp[0] = self.width
        comp.gp[1] = self.height
        comp.gp[2] = self.depth

    def lines(self):
        w, h, d = self.width / 2.0, self.height / 2.0, self.depth / 2.0
        v = [[-w, h, -d], [w, h, -d], [w, -h, -d], [-w, -h, -d],
             [-w, h, d], [w, h, d], [w, -h, d], [-w, -h, d]]
        winding = [0, 1, 2, 3, 0, 4, 5, 1, 2, 6, 5, 6, 7, 4, 0, 3, 7]
        return [[v[i][0] for i in winding], [v[i][1] for i in winding],
                [v[i][2] for i in winding]]
