import numpy as np
import torch

from .sprim import SPrim
from .. import _abi


class SRescal(SPrim):
    """Resolution calculation sample (mcramp/scat/rescal.py:9-65,
    rescal.cl:5-76): the neutron scatters from a random point of its chord
    into a cone of half-angle atan(focus_r/|target|) around ``target``
    (component frame) with final energy E0 +- dE; the event (ki - kf,
    weight, energy transfer) is recorded per neutron index and, after each
    chunk, kept for the neutrons a later component flagged (record lane se,
    set by SCounter), as data_reduce does (rescal.py:47-55).
    Plain path only (one event slot per neutron index of the chunk).
    Slots: sp = target.x, target.y, target.z, E0, dE, focus_r; tally = the
    event buffer (8 floats per neutron index)."""
    kind = _abi.S_RESCAL

    def __init__(self, target=(0, 0, 0), E0=0, dE=0, focus_r=0, idx=0, ctx=None, **kwargs):
        self.idx = np.uint32(idx)
        self.target = np.array(target[:3], dtype=np.float32)
        self.E0 = np.float32(E0)
        self.dE = np.float32(dE)
        self.focus_r = np.float32(focus_r)
        self.events = None
        self.qx_vals = np.array([])
        self.qy_vals = np.array([])
        self.qz_vals = np.array([])
        self.dE_vals = np.array([])
        self.p_vals = np.array([])

    def fill(self, comp, keep):
        super().fill(comp, keep)
        for k, v in enumerate((self.target[0], self.target[1], self.target[2], self.E0, self.dE,
                               self.focus_r)):
            comp.sp[k] = v
        if self.events is not None:
            comp.tally = self.events.data_ptr()
            comp.tally_len = self.events.numel()

    def prepare(self, n, device):
        """Event buffer for chunks of up to n histories on ``device``."""
        if self.events is None or self.events.shape[0] < n or self.events.device != device:
            self.events = torch.zeros((max(int(n), 1), 8), dtype=torch.float32, device=device)
        return self.events

    def begin_chunk(self):
        self.events.zero_()

    def reduce(self, se, n):
        """Keep the events of neutrons [0, n) whose se lane is set."""
        keep = (se[:n] > 0.0)
        ev = self.events[:n][keep].double().cpu().numpy()
        self.qx_vals = np.concatenate((self.qx_vals, ev[:, 0]))
        self.qy_vals = np.concatenate((self.qy_vals, ev[:, 1]))
        self.qz_vals = np.concatenate((self.qz_vals, ev[:, 2]))
        self.dE_vals = np.concatenate((self.dE_vals, ev[:, 7]))
        self.p_vals = np.concatenate((self.p_vals, ev[:, 6]))

    def data(self, queue=None):
        return (self.qx_vals, self.qy_vals, self.qz_vals, self.dE_vals, self.p_vals)
