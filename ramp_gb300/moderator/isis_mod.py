import re

import numpy as np

from .flat_mod import MFlat
from .. import _abi


def _bin_fraction(lower, upper, minimum, maximum):
    """Fraction of the bin [lower, upper] inside [minimum, maximum]
    (isis_mod.py:27-35)."""
    width = upper - lower
    frac = (upper - minimum) / width if minimum > lower else 1.0
    frac -= (upper - maximum) / width if maximum < upper else 0.0
    return frac


_NUM = r"\d*\.\d*[e][+\-]?\d+"
_ROW = re.compile("(?:%s %s \\(%s\\) )" % (_NUM, _NUM, _NUM))


def read_spectrum(path, E_min, E_max):
    """Parse a McStas/MCNP moderator spectrum file (``Let_Base.mcstas``
    format: per energy bin, lines ``t value (error)`` of a time histogram)
    into the tables the MISIS sampler uses (isis_mod.py:85-165):

    flux     cumulative intensity over (energy row, time bin), float32
    t_bins   time-bin values / 1e8 (s), from the first energy block
    e_bins   energy edges in meV: E_min, the bin lower edges inside, E_max
    e_int    cumulative intensity at the energy edges
    total    summed intensity of the rows used
    time_offset  the file's TimeOffset value
    Energy bins partly inside [E_min, E_max] are weighted by the covered
    fraction; the file's energies are in MeV (x 1e9 -> meV as the reference
    does)."""
    with open(path) as f:
        text = f.read()
    lines = text.splitlines(True)
    rows = _ROW.findall(text)
    # first TimeOffset line, then the first line containing "time", then the
    # first line after it containing "total" (line counting as in the
    # reference: num_time_bins = total line - time line - 1)
    k = 0
    while "TimeOffset" not in lines[k]:
        k += 1
    time_offset = np.float32(lines[k].split()[-1])
    t_line = k
    while "time" not in lines[t_line]:
        t_line += 1
    tot_line = t_line
    while "total" not in lines[tot_line]:
        tot_line += 1
    n_t = tot_line - t_line - 1
    e_lo, e_hi = [], []
    for ln in lines:
        if "energy bin" in ln:
            b = re.findall(_NUM, ln)
            e_lo.append(float(b[0]) * 1e9)
            e_hi.append(float(b[1]) * 1e9)
    cells = np.array([r.strip().replace("(", "").replace(")", "") for r in rows])
    cells = cells.reshape(cells.size // n_t, n_t)
    E_min = np.float32(E_min)
    E_max = np.float32(E_max)
    i_lo = int(np.searchsorted(e_lo, E_min))
    i_hi = int(np.searchsorted(e_lo, E_max))
    if E_min == e_lo[0]:
        i_lo += 1
    e_bins = np.array([E_min] + list(e_lo[i_lo:i_hi]) + [E_max])
    fracs = [_bin_fraction(e_lo[i], e_hi[i], E_min, E_max) for i in range(i_lo - 1, i_hi)]
    t_bins = np.array([c.split(" ")[0] for c in cells[0]]).astype(float) / 1e8
    vals = np.array([[c.split(" ")[1] for c in row] for row in cells]).astype(float)
    used = vals[i_lo - 1:i_hi, :] * np.array(fracs)[:, None]
    flux = np.cumsum(used.flatten()).astype(np.float32)
    e_int = np.insert(flux.reshape(used.shape)[:, -1], 0, 0.0).astype(np.float32)
    return dict(flux=flux, t_bins=t_bins.astype(np.float32), e_bins=e_bins.astype(np.float32),
                e_int=e_int, total=np.float32(np.sum(used)), time_offset=time_offset)


def solid_angle_area(mod_dim, target_dim, target_dist, n_steps=50):
    """The source-to-window acceptance integral the reference calls
    str_area (isis_mod.py:45-66): a Riemann sum of 1/r^2 on 50-point grids
    (edges included) over a quarter of the window and the whole moderator
    face, in float64 and in the reference's summation order, times the two
    areas and 1e4."""
    tx = np.linspace(0, target_dim[0] / 2.0, num=n_steps)
    ty = np.linspace(0, target_dim[1] / 2.0, num=n_steps)
    TX, TY = np.meshgrid(tx, ty)
    mx = np.linspace(-mod_dim[0] / 2.0, mod_dim[0] / 2.0, num=n_steps)
    my = np.linspace(-mod_dim[1] / 2.0, mod_dim[1] / 2.0, num=n_steps)
    MX, MY = np.meshgrid(mx, my)
    A = 0.0
    for row_x in MX:
        for row_y in MY:
            A += np.sum(1 / (np.power(-1.0 * TX + row_x, 2.0) + np.power(-1.0 * TY + row_y, 2.0)
                             + target_dist ** 2.0))
    A *= (mod_dim[0] * mod_dim[1]) / (n_steps ** 4.0)
    A *= target_dim[0] * target_dim[1] * 10000
    return np.float32(A)


class MISIS(MFlat):
    """ISIS moderator from a tabulated time-energy spectrum
    (mcramp/moderator/isis_mod.py:10-185, isis_mod.cl:15-104): the flux CDF
    picks a (time, energy) cell, the emission time is interpolated linearly
    inside its time bin and the energy by a 7-point Lagrange polynomial over
    the cumulative flux at the energy edges; direction and spin as MFlat;
    weight str_area * total * 6.2415093e12 / N_chunk, time of flight starting
    at the emission time.  The spectrum file is read once per file and
    energy range."""
    kind = _abi.SRC_ISIS
    _cache = {}

    def __init__(self, ctx=None, spec_file="Let_Base.mcstas", mod_dim=(0.0, 0.0),
                 target_dim=(0.0, 0.0), target_dist=0.0, E_min=0.0, E_max=0.0):
        super().__init__(ctx, spec_file, mod_dim, target_dim, target_dist, E_min, E_max)
        key = (spec_file, float(self.E_min), float(self.E_max))
        if key not in MISIS._cache:
            MISIS._cache[key] = read_spectrum(spec_file, E_min, E_max)
        self.spectrum = MISIS._cache[key]
        self.total = self.spectrum["total"]
        self.time_offset = self.spectrum["time_offset"]
        self.str_area = solid_angle_area(mod_dim, target_dim, target_dist)

    def params(self):
        return super().params() + [0.0] * 6 + [self.str_area, self.total]

    def descriptor(self):
        s = super().descriptor()
        sp = self.spectrum
        self._tables = [np.ascontiguousarray(sp[k], dtype=np.float32)
                        for k in ("flux", "t_bins", "e_bins", "e_int")]
        for k, t in enumerate(self._tables):
            s.table[k] = t.ctypes.data_as(_abi.ctypes.POINTER(_abi.ctypes.c_float))
            s.table_len[k] = t.size
        return s
