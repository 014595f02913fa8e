import datetime

import numpy as np
import torch

from .sprim import SPrim, _device
from .. import _abi

_GRIDS = {}   # (binnings, bin counts) -> (X, Y) coordinate grids

VAR_DICT = {"x": 0, "y": 1, "theta": 2, "alpha": 3, "phi": 4, "tof": 5, "divX": 6, "divY": 7,
            "wavelength": 8, "energy": 9, "angle": 10}


class SDetector2D(SPrim):
    """Two-axis histogram monitor (mcramp/scat/detector2D.py:11-207,
    detector2D.cl:3-186).  Bin = round((v-min)/step) for min <= v <= max,
    n = ceil((max-min)/step), flat index i1*n2 + i2; the top half-bin maps
    to index n, which inside the buffer lands in the next row (kept, as in
    the reference) and past its end is dropped and counted.  data() returns
    (X, Y, Z, E) with Z = histogram.reshape(n1, n2).T.
    Slots: sp[0..2], sp[3..5] = axis binnings, si[0], si[1] = axis vars,
    si[2], si[3] = n1, n2, si[4] = restore."""
    kind = _abi.S_DET2D

    def __init__(self, shape="", axis1_binning=(0, 0, 0), axis2_binning=(0, 0, 0),
                 axis1_var="theta", axis2_var="tof", restore_neutron=False, idx=0, ctx=None,
                 filename=None, logscale=False, **kwargs):
        self.var_label_dict = {0: "x [m]", 1: "y [m]", 2: "Theta [deg]", 3: "Alpha [deg]",
                               4: "Phi [deg]", 5: "Time-of-flight [us]",
                               6: "Horizontal divergence [deg]", 7: "Vertical divergence [deg]",
                               8: "Wavelength [Ang]", 9: "Energy [meV]", 10: "Bragg angle [deg]"}
        self.axis1_var = np.uint32(VAR_DICT[axis1_var])
        self.axis2_var = np.uint32(VAR_DICT[axis2_var])
        if not (axis1_binning[1] > 0 and axis2_binning[1] > 0):
            raise ValueError("SDetector2D binning steps must be positive")
        self.axis1_binning = np.array(axis1_binning[:3], dtype=np.float32)
        self.axis2_binning = np.array(axis2_binning[:3], dtype=np.float32)
        self.idx = np.uint32(idx)
        self.restore_neutron = np.uint32(1 if restore_neutron else 0)
        self.filename = filename
        self.logscale = logscale
        self.axis1_num_bins = np.uint32(np.ceil((axis1_binning[2] - axis1_binning[0]) /
                                                axis1_binning[1]))
        self.axis2_num_bins = np.uint32(np.ceil((axis2_binning[2] - axis2_binning[0]) /
                                                axis2_binning[1]))
        self.num_bins = np.uint32(self.axis1_num_bins * self.axis2_num_bins)
        dev = _device(ctx)
        self.histo_t = torch.zeros(int(self.num_bins), dtype=torch.float32, device=dev)
        self.histo_err_t = torch.zeros(int(self.num_bins), dtype=torch.float32, device=dev)
        self._XY = None
        self.last_ran_datetime = datetime.datetime.now()

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.sp[0], comp.sp[1], comp.sp[2] = self.axis1_binning
        comp.sp[3], comp.sp[4], comp.sp[5] = self.axis2_binning
        comp.si[0] = int(self.axis1_var)
        comp.si[1] = int(self.axis2_var)
        comp.si[2] = int(self.axis1_num_bins)
        comp.si[3] = int(self.axis2_num_bins)
        comp.si[4] = int(self.restore_neutron)
        comp.tally = self.histo_t.data_ptr()
        comp.tally_err = self.histo_err_t.data_ptr()
        comp.tally_len = int(self.num_bins)

    def tallies(self):
        return [self.histo_t, self.histo_err_t]

    def _grid(self):
        # bin-coordinate grids (two n2 x n1 float64 arrays), built once per
        # binning in the process and shared read-only by every detector
        if self._XY is None:
            key = (tuple(self.axis1_binning.tolist()), int(self.axis1_num_bins),
                   tuple(self.axis2_binning.tolist()), int(self.axis2_num_bins))
            XY = _GRIDS.get(key)
            if XY is None:
                x = np.linspace(self.axis1_binning[0], self.axis1_binning[2],
                                num=int(self.axis1_num_bins))
                y = np.linspace(self.axis2_binning[0], self.axis2_binning[2],
                                num=int(self.axis2_num_bins))
                XY = np.meshgrid(x, y)
                for g in XY:
                    g.setflags(write=False)
                _GRIDS[key] = XY
            self._XY = XY
        return self._XY

    @property
    def X(self):
        return self._grid()[0]

    @property
    def Y(self):
        return self._grid()[1]

    @property
    def histo(self):
        return self.histo_t.cpu().numpy()

    @property
    def histo_err(self):
        return self.histo_err_t.cpu().numpy()

    @property
    def Z(self):
        return self.histo.reshape((int(self.axis1_num_bins), int(self.axis2_num_bins))).T

    @property
    def E(self):
        return self.histo_err.reshape((int(self.axis1_num_bins), int(self.axis2_num_bins))).T

    def data(self, queue=None):
        return (self.X, self.Y, self.Z, self.E)

    def get_histo(self):
        return self.data()

    def save(self, queue=None):
        if self.filename:
            np.save(self.filename + 'X', self.X)
            np.save(self.filename + 'Y', self.Y)
            np.save(self.filename + 'Z', self.Z)
            np.save(self.filename + 'E', self.E)

    def plot(self, queue=None):
        import matplotlib.pyplot as plt
        Z = np.log(self.Z + 1e-7) if self.logscale else self.Z
        plt.figure()
        plt.pcolormesh(self.X, self.Y, Z, cmap='jet', shading='auto')
        plt.xlabel(self.var_label_dict[int(self.axis1_var)])
        plt.ylabel(self.var_label_dict[int(self.axis2_var)])
        plt.colorbar()
        plt.tight_layout()
