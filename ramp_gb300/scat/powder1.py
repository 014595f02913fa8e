import numpy as np

from .sprim import SPrim
from .. import _abi


class SPowder1(SPrim):
    """Single-line Bragg powder (mcramp/scat/powder1.py:9-80, powder1.cl:
    5-100): a neutron that can satisfy the Bragg condition scatters onto
    the Debye-Scherrer cone (phi focusing over +-d_phi degrees on both
    sides of the beam), at a depth drawn from the attenuation.  Host
    preparation as powder1.py:53-62, in float64 then rounded:
    q = 2 pi / d, sigma v^2 = 4 pi^3 pack mult F2 100 DW / (vc^2 q),
    sigma_abs v = pack sigma_abs / vc * 100.
    Slots: sp = sigma_scat*v^2, sigma_abs*v, q, d_phi."""
    kind = _abi.S_POWDER1

    def __init__(self, d_spacing=0.0, pack=0.0, vc=0.0, sigma_abs=0.0, multiplicity=0, DW=0.0,
                 F2=0.0, d_phi=180.0, idx=0, ctx=None, **kwargs):
        q = (2 * np.pi) / d_spacing
        numer = 4 * np.pi ** 3.0 * pack * multiplicity * F2 * 100 * DW
        denom = vc ** 2.0 * q
        self.sigma_scat_v2 = np.float32(numer / denom)
        self.sigma_abs_v = np.float32(pack * sigma_abs / vc * 100)
        self.q = np.float32(q)
        self.idx = np.uint32(idx)
        self.d_phi = np.float32(d_phi)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.sp[0] = self.sigma_scat_v2
        comp.sp[1] = self.sigma_abs_v
        comp.sp[2] = self.q
        comp.sp[3] = self.d_phi
