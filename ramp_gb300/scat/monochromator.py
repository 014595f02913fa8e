import numpy as np

from .sprim import SPrim
from .. import _abi


def gauss_legendre_15():
    """Nodes and weights of 15-point Gauss-Legendre quadrature on [-1, 1]
    (float32), the normalisation rule of the monochromator mosaic."""
    x, w = np.polynomial.legendre.leggauss(15)
    return x.astype(np.float32), w.astype(np.float32)


class SMonochromator(SPrim):
    """Mosaic crystal monochromator, flat or curved (mcramp/scat/
    monochromator.py:10-111, monochromator.cl:22-195): reflection from the
    local yz plane, higher orders, anisotropic Gaussian mosaic (arc
    minutes), n_horizontal x n_vertical slabs with gaps, curvature radii.
    Slots: sp = slab_width, slab_height, gap, mosaic_horizontal,
    mosaic_vertical, r0, d_spacing, radius_vertical, radius_horizontal;
    si = n_horizontal, n_vertical; table[0], table[1] = Gauss-Legendre
    nodes and weights."""
    kind = _abi.S_MONO

    def __init__(self, slab_width=0.0, slab_height=0.0, gap=0.0, n_horizontal=1, n_vertical=1,
                 mosaic_horizontal=0.0, mosaic_vertical=0.0, r0=1.0, d_spacing=0.0,
                 radius_vertical=0.0, radius_horizontal=0.0, idx=0, ctx=0, **kwargs):
        self.gauss_x, self.gauss_w = gauss_legendre_15()
        self.idx = np.uint32(idx)
        self.slab_width = np.float32(slab_width)
        self.slab_height = np.float32(slab_height)
        self.gap = np.float32(gap)
        self.n_horizontal = np.uint32(n_horizontal)
        self.n_vertical = np.uint32(n_vertical)
        self.mosaic_horizontal = np.float32(mosaic_horizontal)
        self.mosaic_vertical = np.float32(mosaic_vertical)
        self.r0 = np.float32(r0)
        self.d_spacing = np.float32(d_spacing)
        self.radius_vertical = np.float32(radius_vertical)
        self.radius_horizontal = np.float32(radius_horizontal)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        for k, v in enumerate((self.slab_width, self.slab_height, self.gap,
                               self.mosaic_horizontal, self.mosaic_vertical, self.r0,
                               self.d_spacing, self.radius_vertical, self.radius_horizontal)):
            comp.sp[k] = v
        comp.si[0] = int(self.n_horizontal)
        comp.si[1] = int(self.n_vertical)
        _abi.set_table(comp, 0, self.gauss_x, keep)
        _abi.set_table(comp, 1, self.gauss_w, keep)
