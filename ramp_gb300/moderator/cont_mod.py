import numpy as np

from .flat_mod import MFlat
from .. import _abi


class MCont(MFlat):
    """Continuous three-Maxwellian moderator (mcramp/moderator/cont_mod.py:
    10-70, cont_mod.cl:4-73): as MFlat, with weight
    sum_i I_i M(E; T_i) / M(k_B T_i; T_i) / N_chunk.  Any T_i = 0 gives a NaN
    weight as in the reference, so a single-temperature source sets
    T1 = T2 = T3 with I2 = I3 = 0.  str_area is fixed at 1 (cont_mod.py:30)."""
    kind = _abi.SRC_CONT

    def __init__(self, ctx=None, spec_file="Let_Base.mcstas", mod_dim=(0.0, 0.0),
                 target_dim=(0.0, 0.0), target_dist=0.0, E_min=0.0, E_max=0.0, T1=0.0, I1=0.0,
                 T2=0.0, I2=0.0, T3=0.0, I3=0.0):
        super().__init__(ctx, spec_file, mod_dim, target_dim, target_dist, E_min, E_max)
        self.T1, self.I1, self.T2, self.I2, self.T3, self.I3 = (
            np.float32(v) for v in (T1, I1, T2, I2, T3, I3))
        self.str_area = np.float32(1)

    def params(self):
        return super().params() + [self.T1, self.I1, self.T2, self.I2, self.T3, self.I3,
                                   self.str_area]
