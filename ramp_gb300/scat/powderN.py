import numpy as np

from .sprim import SPrim
from .. import _abi


class SPowderN(SPrim):
    """Bragg powder with N lines (mcramp/scat/powderN.py:9-91,
    powderN.cl:5-157).  Host preparation as powderN.py:59-72:
    q_i = 2 pi / d_i, sigma_i v^2 = 4 pi^3 pack mult F2 100 DW / (vc^2 q_i),
    sigma_abs v = pack sigma_abs / vc * 100.
    Slots: table[0] = sigma_scat*v^2, table[1] = q, sp[0] = sigma_abs*v,
    sp[1] = d_phi, si[0] = num_lines, si[1] = transmit."""
    kind = _abi.S_POWDERN

    def __init__(self, d_spacing=[0.0], pack=0.0, vc=0.0, sigma_abs=0.0, multiplicity=[0],
                 DW=0.0, F2=[0.0], d_phi=180.0, transmit=1, idx=0, ctx=None, **kwargs):
        self.d_spacing = np.asarray(d_spacing, dtype=np.float64)
        self.pack, self.vc, self.sigma_abs, self.DW = pack, vc, sigma_abs, DW
        self.multiplicity = np.asarray(multiplicity)
        self.F2 = np.asarray(F2, dtype=np.float64)
        q = np.array((2 * np.pi) / self.d_spacing, dtype=np.float32)
        numer = np.array(4 * np.pi ** 3.0 * pack * self.multiplicity * self.F2 * 100 * DW,
                         dtype=np.float32)
        denom = np.float32(vc ** 2.0) * q
        self.q = q
        self.sigma_scat_v2 = (numer / denom).astype(np.float32)
        self.sigma_abs_v = np.float32(pack * sigma_abs / vc * 100) if vc else np.float32(0)
        self.idx = np.uint32(idx)
        self.d_phi = np.float32(d_phi)
        self.num_lines = np.uint32(len(self.d_spacing))
        self.transmit = np.uint32(transmit)
        if self.num_lines < 1:
            raise ValueError("SPowderN needs at least one line")

    def fill(self, comp, keep):
        super().fill(comp, keep)
        _abi.set_table(comp, 0, self.sigma_scat_v2, keep)
        _abi.set_table(comp, 1, self.q, keep)
        comp.sp[0] = self.sigma_abs_v
        comp.sp[1] = self.d_phi
        comp.si[0] = int(self.num_lines)
        comp.si[1] = int(self.transmit)
