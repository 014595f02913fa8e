import datetime

import numpy as np
import torch

from .sprim import SPrim, _device
from .. import _abi


class SDetector1D(SPrim):
    """One-axis histogram monitor (mcramp/scat/detector1D.py:11-138,
    detector1D.cl:20-77).  var: energy, theta, tof [us] or wavelength; bin
    = floor((v-min)/step) for min <= v <= max, n = ceil((max-min)/step);
    the top edge maps to index n, which the reference writes past its
    buffer: here that write is dropped and counted.  Accumulates sum(p) and
    sum(p^2).  Slots: sp[0..2] = binning, si[0] = var, si[1] = restore,
    si[2] = n_bins; tally/tally_err = histogram, squared-weight histogram."""
    kind = _abi.S_DET1D

    def __init__(self, binning=(0, 0, 0), logscale=False, restore_neutron=False, idx=0,
                 var="energy", ctx=None, filename=None, **kwargs):
        var_dict = {"energy": 0, "theta": 1, "tof": 2, "wavelength": 3}
        self.var_label_dict = {0: "Energy [meV]", 1: "Theta [deg]", 2: "Time-of-flight [us]",
                               3: "Wavelength [Ang]"}
        self.var = np.uint32(var_dict[var])
        if not binning[1] > 0:
            raise ValueError("SDetector1D binning step must be positive")
        self.binning = np.array((binning[0], binning[1], binning[2]), dtype=np.float32)
        self.idx = idx
        self.logscale = logscale
        self.num_bins = np.uint32(np.ceil((binning[2] - binning[0]) / binning[1]))
        self.restore = np.uint32(1 if restore_neutron else 0)
        self.filename = filename
        dev = _device(ctx)
        self.histo_t = torch.zeros(int(self.num_bins), dtype=torch.float32, device=dev)
        self.histo_err_t = torch.zeros(int(self.num_bins), dtype=torch.float32, device=dev)
        self.axis = np.linspace(self.binning[0], self.binning[2], num=int(self.num_bins))
        self.last_ran_datetime = datetime.datetime.now()

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.sp[0], comp.sp[1], comp.sp[2] = self.binning
        comp.si[0] = int(self.var)
        comp.si[1] = int(self.restore)
        comp.si[2] = int(self.num_bins)
        comp.tally = self.histo_t.data_ptr()
        comp.tally_err = self.histo_err_t.data_ptr()
        comp.tally_len = int(self.num_bins)

    def tallies(self):
        return [self.histo_t, self.histo_err_t]

    @property
    def histo(self):
        h = self.histo_t.cpu().numpy().copy()
        h[np.isnan(h)] = 0
        return h

    @property
    def histo_err(self):
        h = self.histo_err_t.cpu().numpy().copy()
        h[np.isnan(h)] = 0
        return h

    def data(self, queue=None):
        return (self.axis, self.histo, self.histo_err)

    def get_histo(self):
        return self.data()

    def save(self, queue=None):
        if self.filename:
            np.save(self.filename + 'X', self.axis)
            np.save(self.filename + 'Y', self.histo)
            np.save(self.filename + 'E', self.histo_err)

    def plot(self, queue=None):
        import matplotlib.pyplot as plt
        h = self.histo
        plt.figure()
        plt.errorbar(self.axis, np.log(h + 1e-7) if self.logscale else h,
                     np.sqrt(self.histo_err), capsize=8)
        plt.ylabel("Intensity")
        plt.xlabel(self.var_label_dict[int(self.var)])
        plt.tight_layout()
