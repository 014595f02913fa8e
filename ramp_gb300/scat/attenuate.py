import numpy as np

from .sprim import SPrim
from .. import _abi


class SAttenuate(SPrim):
    """Constant-mu attenuator for mesh imaging.  No reference counterpart
    (RAMP has no constant-mu absorber): paired with a GMesh geometry, the
    neutron weight is multiplied by exp(-mu * L), L the summed length of
    all chords the ray cuts through the mesh (crossings sorted along the
    ray, each entry paired with the next exit, repeated crossings at shared
    edges ignored; the ray starts outside the mesh), and the neutron is
    moved to the earliest exit point.  ``mu`` is in 1/m.  Slots: sp[0] = mu."""
    kind = _abi.S_ATTENUATE

    def __init__(self, mu=0.0, idx=0, ctx=None, **kwargs):
        self.mu = np.float32(mu)
        self.idx = np.uint32(idx)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.sp[0] = self.mu
