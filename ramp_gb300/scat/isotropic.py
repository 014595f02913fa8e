import re

import numpy as np

from .sprim import SPrim
from .. import _abi


def simps(y, x, axis=-1):
    """Composite Simpson integral of samples y(x) on an irregular grid, with
    the 'avg' treatment of an even sample count (the behaviour of
    scipy.integrate.simps that the reference's table preparation calls,
    isotropic.py:7,201-211; that function is gone from current SciPy).
    One sample integrates to 0, two samples to the trapezoid."""
    y = np.asarray(y, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    y = np.moveaxis(y, axis, -1)
    n = y.shape[-1]
    if n < 2:
        return np.zeros(y.shape[:-1])

    def basic(yy, xx):
        m = yy.shape[-1]
        if m < 2:
            return np.zeros(yy.shape[:-1])
        if m < 3:
            return 0.5 * (xx[1] - xx[0]) * (yy[..., 0] + yy[..., 1])
        h = np.diff(xx)
        h0, h1 = h[0:m - 2:2], h[1:m - 1:2]
        hs, hp, hq = h0 + h1, h0 * h1, h0 / h1
        t = yy[..., 0:m - 2:2] * (2.0 - 1.0 / hq) + yy[..., 1:m - 1:2] * (hs * hs / hp) \
            + yy[..., 2:m:2] * (2.0 - hq)
        return np.sum(hs / 6.0 * t, axis=-1)

    if n % 2 == 1:
        return basic(y, x)
    first = basic(y[..., :-1], x[:-1]) + 0.5 * (x[-1] - x[-2]) * (y[..., -1] + y[..., -2])
    last = basic(y[..., 1:], x[1:]) + 0.5 * (x[1] - x[0]) * (y[..., 0] + y[..., 1])
    return 0.5 * (first + last)


def cdf_from_pd(x, pd):
    """Normalised running integral (mcramp/scat/isotropic.py:210-212)."""
    unnormed = np.array([simps(pd[:i], x=x[:i]) for i in range(1, len(x) + 1)],
                        dtype=np.float32)
    return unnormed / unnormed[-1]


def load_sqw(fn):
    """Parse a McStas Isotropic_Sqw file as mcramp/scat/isotropic.py:171-208
    does, quirks included: the last q value is dropped, the first S(q,w)
    row is consumed by the header loop, sigma_scat is read from the
    ``sigma_coh`` header field and machine epsilon is added to S."""
    header = {}
    flag = 0
    q = w = None
    with open(fn, "r") as fin:
        for line in fin:
            data = re.findall(r"#\s+([A-za-z_]+)\s+([-+]?\d*\.\d+|\d+)", line)
            if data:
                header[data[0][0]] = data[0][1]
            if not line[0] == "#":
                if flag == 0:
                    q = np.array(line.split(), dtype=np.float32)[:-1]
                    flag += 1
                    continue
                elif flag == 1:
                    w = np.array(line.split(), dtype=np.float32)
                    flag += 1
                    continue
                else:
                    break
        rows = [r for r in (l.split() for l in fin.readlines()) if r and not r[0].startswith("#")]
    sqw = np.array(rows, dtype=np.float64).astype(np.float32) + np.float32(np.finfo(float).eps)
    sigma_abs = np.float32(header["sigma_abs"])
    sigma_coh = np.float32(header["sigma_coh"])
    rho = np.float32(header["V_rho"])
    sigma_scat = sigma_coh
    pw = simps(q * sqw.T, axis=1, x=q)
    pw /= simps(pw, x=w)
    norm = simps(sqw.T, axis=0, x=w)
    pq = np.array([q * sqw[:, i] / norm for i in range(0, len(w))])
    pw_cdf = cdf_from_pd(w, pw)
    pq_cdf = np.array([cdf_from_pd(q, pq[j, :]) for j in range(0, len(w))], dtype=np.float32)
    return q, w, rho, sigma_abs, sigma_scat, pw_cdf, pq_cdf, sqw


class SIsotropic(SPrim):
    """Isotropic S(Q,w) scatterer with coherent, incoherent and magnetic
    channels and 1/v absorption (mcramp/scat/isotropic.py:12-212,
    isotropic.cl:5-323).
    Slots per channel c (0 coh, 1 inc, 2 mag): table[4c..4c+3] = q, w,
    pw_cdf, pq_cdf (flattened [n_w, n_q]); sp[1+3c..3+3c] = rho, sigma_abs,
    sigma_scat; si[1+2c], si[2+2c] = n_q, n_w.  sp[0] = temperature,
    si[0] = transmit."""
    kind = _abi.S_ISOTROPIC

    def __init__(self, fn_coh='', fn_inc='', fn_mag='', temperature=0, transmit=1, idx=0,
                 ctx=None, **kwargs):
        self.temperature = np.float32(temperature)
        self.transmit = np.uint32(transmit)
        if fn_coh == '' and fn_inc == '' and fn_mag == '':
            raise ValueError("Invalid filename combination")
        self.idx = np.uint32(idx)
        self.channels = []
        for fn in (fn_coh, fn_inc, fn_mag):
            if fn:
                q, w, rho, sa, ss, pw_cdf, pq_cdf, _ = load_sqw(fn)
                self.channels.append((q, w, pw_cdf, pq_cdf.ravel(), rho, sa, ss, True))
            else:
                z = np.zeros(1, dtype=np.float32)
                self.channels.append((z, z, z, z, np.float32(0), np.float32(0), np.float32(0),
                                      False))

    def fill(self, comp, keep):
        super().fill(comp, keep)
        comp.sp[0] = self.temperature
        comp.si[0] = int(self.transmit)
        for c, (q, w, pw_cdf, pq_cdf, rho, sa, ss, present) in enumerate(self.channels):
            for j, t in enumerate((q, w, pw_cdf, pq_cdf)):
                _abi.set_table(comp, 4 * c + j, t, keep)
            comp.sp[1 + 3 * c] = rho
            comp.sp[2 + 3 * c] = sa
            comp.sp[3 + 3 * c] = ss
            comp.si[1 + 2 * c] = len(q) if present else 0
            comp.si[2 + 2 * c] = len(w) if present else 0
