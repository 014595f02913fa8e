"""MCPL particle files (Monte Carlo Particle Lists, format version 3).

Reader and writer for the subset RAMP exchanges with McStas/Geant4:
neutrons (PDG 2112), single or double precision, optional polarisation,
per-particle or universal PDG code and weight, optional user flags,
comments and binary blobs (skipped), gzip-compressed files.  Units as in
MCPL: position cm, kinetic energy MeV, time ms.

Directions are packed into two numbers and the sign of the kinetic-energy
field by the adaptive projection of the MCPL paper (T. Kittelmann et al.,
"Monte Carlo Particle Lists: MCPL", Comput. Phys. Commun. 218 (2017)
17-42): with |z| largest the file holds (x, y); with |y| largest
(x, 1/z); with |x| largest (1/z, y); the sign of the largest component is
the sign of the energy field.  ``write(..., packing="ramp")`` reproduces
instead, byte for byte, what RAMP's SMCPLOut writes (mcpl_out.py:7-81: its
own packing, single precision, polarisation, universal PDG 2112, source
name "RAMP"), which standard readers do not decode into the original
directions.
"""
import gzip
import struct

import numpy as np

MAGIC = b"MCPL"


def _open(path, mode):
    return gzip.open(path, mode) if str(path).endswith(".gz") else open(path, mode)


def read(path):
    """Particles of an MCPL file as a dict of numpy arrays: x, y, z (cm),
    ux, uy, uz, ekin (MeV), time (ms), weight, polx, poly, polz, pdgcode,
    userflags."""
    with _open(path, "rb") as f:
        b = f.read()
    if b[:4] != MAGIC:
        raise ValueError("%s is not an MCPL file" % path)
    version = int(b[4:7])
    if version not in (2, 3):
        raise ValueError("MCPL format version %d is not supported" % version)
    if b[7:8] != b"L":
        raise ValueError("big-endian MCPL files are not supported")
    off = 8
    n, = struct.unpack_from("<Q", b, off)
    off += 8
    ncomments, nblobs, userflags, pol, single, pdg, psize, univ_w = struct.unpack_from("<8I", b, off)
    off += 32
    pdg = struct.unpack("<i", struct.pack("<I", pdg))[0]
    weight_u = None
    if univ_w:
        weight_u, = struct.unpack_from("<d", b, off)
        off += 8
    ln, = struct.unpack_from("<I", b, off)
    off += 4 + ln                                  # source name
    for _ in range(ncomments):
        ln, = struct.unpack_from("<I", b, off)
        off += 4 + ln
    for _ in range(nblobs):                        # keys, then data
        ln, = struct.unpack_from("<I", b, off)
        off += 4 + ln
    for _ in range(nblobs):
        ln, = struct.unpack_from("<I", b, off)
        off += 4 + ln
    ft = np.dtype("<f4") if single else np.dtype("<f8")
    fields = []
    if pol:
        fields += [("polx", ft), ("poly", ft), ("polz", ft)]
    fields += [("x", ft), ("y", ft), ("z", ft), ("d0", ft), ("d1", ft), ("ek", ft), ("time", ft)]
    if not univ_w:
        fields.append(("weight", ft))
    if pdg == 0:
        fields.append(("pdgcode", "<i4"))
    if userflags:
        fields.append(("userflags", "<u4"))
    dt = np.dtype(fields)
    if dt.itemsize != psize:
        raise ValueError("particle size %d does not match the header's options (%d)"
                         % (psize, dt.itemsize))
    rec = np.frombuffer(b, dtype=dt, count=n, offset=off)
    d0 = rec["d0"].astype(np.float64)
    d1 = rec["d1"].astype(np.float64)
    ek = rec["ek"].astype(np.float64)
    sign = np.where(np.signbit(ek), -1.0, 1.0)
    ux, uy, uz = d0.copy(), d1.copy(), np.zeros(n)
    xbig = np.abs(d0) > 1.0
    ybig = ~xbig & (np.abs(d1) > 1.0)
    zbig = ~xbig & ~ybig
    with np.errstate(divide="ignore", invalid="ignore"):
        uz[xbig] = 1.0 / d0[xbig]
        ux[xbig] = sign[xbig] * np.sqrt(np.clip(1.0 - d1[xbig] ** 2 - uz[xbig] ** 2, 0.0, None))
        uz[ybig] = 1.0 / d1[ybig]
        uy[ybig] = sign[ybig] * np.sqrt(np.clip(1.0 - d0[ybig] ** 2 - uz[ybig] ** 2, 0.0, None))
        uz[zbig] = sign[zbig] * np.sqrt(np.clip(1.0 - d0[zbig] ** 2 - d1[zbig] ** 2, 0.0, None))
    out = dict(x=rec["x"].astype(np.float64), y=rec["y"].astype(np.float64),
               z=rec["z"].astype(np.float64), ux=ux, uy=uy, uz=uz, ekin=np.abs(ek),
               time=rec["time"].astype(np.float64))
    out["weight"] = (np.full(n, weight_u) if univ_w else rec["weight"].astype(np.float64))
    for k in ("polx", "poly", "polz"):
        out[k] = rec[k].astype(np.float64) if pol else np.zeros(n)
    out["pdgcode"] = rec["pdgcode"].copy() if pdg == 0 else np.full(n, pdg, dtype=np.int32)
    out["userflags"] = rec["userflags"].copy() if userflags else np.zeros(n, dtype=np.uint32)
    return out


def _header(count, source=b"RAMP"):
    return (MAGIC + b"003" + b"L" + struct.pack("<Q", count) +
            struct.pack("<8I", 0, 0, 0, 1, 1, 2112, 44, 0) + struct.pack("<I", len(source)) +
            source)


def _pack_ramp(v):
    """mcpl_out.py:37-55 on float32 velocity rows: (1/vz, 0, sign vx) when
    vx is the largest signed component, (vx, 1/vz, sign vy) when vy is,
    (0, 0, sign vz) when vz is, else (0, 0, 1)."""
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    one = np.float32(1.0)
    zero = np.zeros_like(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv_z = one / z
    cx = (x > y) & (x > z)
    cy = ~cx & (y > x) & (y > z)
    cz = ~cx & ~cy & (z > x) & (z > y)
    ux = np.where(cx, inv_z, np.where(cy, x, zero))
    uy = np.where(cy, inv_z, zero)
    si = np.where(cx, np.sign(x), np.where(cy, np.sign(y), np.where(cz, np.sign(z), one)))
    return ux.astype(np.float32), uy.astype(np.float32), si.astype(np.float32)


def write(path, pos, vel, pol, tof, weight, packing="mcpl", source=b"RAMP"):
    """Write neutrons given in RAMP units (position m, velocity m/s, time of
    flight s, float32 arrays of n rows) as an MCPL file: single precision,
    polarisation, universal PDG 2112."""
    pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3)
    vel = np.asarray(vel, dtype=np.float32).reshape(-1, 3)
    pol = np.asarray(pol, dtype=np.float32).reshape(-1, 3)
    tof = np.asarray(tof, dtype=np.float32).reshape(-1)
    weight = np.asarray(weight, dtype=np.float32).reshape(-1)
    n = pos.shape[0]
    rec = np.zeros((n, 11), dtype=np.float32)
    rec[:, 0:3] = pol
    rec[:, 3:6] = pos * np.float32(1e2)
    if packing == "ramp":
        ux, uy, si = _pack_ramp(vel)
        vm2 = vel[:, 0] * vel[:, 0] + vel[:, 1] * vel[:, 1] + vel[:, 2] * vel[:, 2]
        ke = np.float32(5.22703725e-15) * vm2
        rec[:, 6], rec[:, 7], rec[:, 8] = ux, uy, si * ke
    elif packing == "mcpl":
        v = vel.astype(np.float64)
        speed = np.sqrt((v * v).sum(axis=1))
        with np.errstate(divide="ignore", invalid="ignore"):
            u = v / speed[:, None]
        ek = 5.22703725e-15 * speed * speed           # m/s -> MeV
        a = np.abs(u)
        xbig = (a[:, 0] > a[:, 1]) & (a[:, 0] > a[:, 2])
        ybig = ~xbig & (a[:, 1] > a[:, 2])
        with np.errstate(divide="ignore"):
            inv_z = 1.0 / u[:, 2]
        d0 = np.where(xbig, inv_z, u[:, 0])
        d1 = np.where(ybig, inv_z, u[:, 1])
        big = np.where(xbig, u[:, 0], np.where(ybig, u[:, 1], u[:, 2]))
        rec[:, 6], rec[:, 7] = d0, d1
        rec[:, 8] = np.where(big < 0, -ek, ek)
    else:
        raise ValueError("packing must be 'mcpl' or 'ramp'")
    rec[:, 9] = tof * np.float32(1e3)
    rec[:, 10] = weight
    with _open(path, "wb") as f:
        f.write(_header(n, source))
        f.write(rec.tobytes())
