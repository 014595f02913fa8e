from random import randint

import numpy as np

from .. import _abi


class MFlat:
    """Flat-spectrum moderator (mcramp/moderator/flat_mod.py:10-32,
    flat_mod.cl:4-51): energy uniform in [E_min, E_max] (uniform in energy,
    not wavelength), start point uniform on the moderator rectangle,
    direction towards a uniform point of the target window at target_dist,
    spin uniform on the sphere, weight 1/N_chunk.  ``spec_file`` is accepted
    and unused, as in the reference."""
    kind = _abi.SRC_FLAT

    def __init__(self, ctx=None, spec_file="Let_Base.mcstas", mod_dim=(0.0, 0.0),
                 target_dim=(0.0, 0.0), target_dist=0.0, E_min=0.0, E_max=0.0):
        self.mod_dim = np.array(mod_dim[:2], dtype=np.float32)
        self.target_dim = np.array(target_dim[:2], dtype=np.float32)
        self.target_dist = np.float32(target_dist)
        self.E_min = np.float32(E_min)
        self.E_max = np.float32(E_max)

    def params(self):
        return [self.mod_dim[0], self.mod_dim[1], self.target_dim[0], self.target_dim[1],
                self.target_dist, self.E_min, self.E_max]

    def descriptor(self):
        s = _abi.RampSource()
        s.kind = self.kind
        for k, v in enumerate(self.params()):
            s.p[k] = v
        return s

    def next_seed(self):
        """The per-chunk seed, drawn exactly as gen_prg does
        (flat_mod.py:32: random.randint(0, 4096))."""
        return int(np.int32(randint(0, 4096)))

    def gen_prg(self, queue, N, neutron_buf, intersection_buf=None):
        raise NotImplementedError("moderators run through Instrument.execute")
