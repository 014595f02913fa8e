import os
import struct

import numpy as np

from .gprim import GPrim
from .. import _abi


_STL_CACHE = {}


def read_stl_cached(filename):
    """read_stl with a per-process cache keyed by path and modification
    time: components built from the same file share one (read-only) array."""
    key = (os.path.abspath(filename), os.path.getmtime(filename))
    pts = _STL_CACHE.get(key)
    if pts is None:
        pts = read_stl(filename)
        pts.setflags(write=False)
        _STL_CACHE[key] = pts
    return pts


def read_stl(filename):
    """Triangles of an STL file (binary or ASCII) as a float32 array
    [n_tri, 9] = v0, v1, v2, the layout numpy-stl's ``mesh.points`` gives
    (mcramp/geom/mesh.py:63-73)."""
    with open(filename, "rb") as f:
        data = f.read()
    if len(data) >= 84:
        n = struct.unpack_from("<I", data, 80)[0]
        if 84 + 50 * n == len(data):
            rec = np.dtype([("normal", "<f4", 3), ("v", "<f4", 9), ("attr", "<u2")])
            tri = np.frombuffer(data, dtype=rec, count=n, offset=84)
            return np.ascontiguousarray(tri["v"], dtype=np.float32)
    text = data.decode("ascii", errors="replace").split()
    verts = []
    i = 0
    while i < len(text):
        if text[i] == "vertex":
            verts.extend((float(text[i + 1]), float(text[i + 2]), float(text[i + 3])))
            i += 4
        else:
            i += 1
    if len(verts) % 9:
        raise ValueError("malformed STL file %s" % filename)
    return np.asarray(verts, dtype=np.float32).reshape(-1, 9)


def write_stl(filename, tris):
    """Write float32 triangles [n, 9] as a binary STL (normals computed)."""
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    v0, v1, v2 = tris[:, 0:3], tris[:, 3:6], tris[:, 6:9]
    nrm = np.cross(v1 - v0, v2 - v0)
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = (nrm / np.where(ln == 0, 1, ln)).astype(np.float32)
    rec = np.zeros(len(tris), dtype=np.dtype([("normal", "<f4", 3), ("v", "<f4", 9),
                                              ("attr", "<u2")]))
    rec["normal"] = nrm
    rec["v"] = tris
    with open(filename, "wb") as f:
        f.write(b"ramp_gb300 binary STL".ljust(80, b" "))
        f.write(struct.pack("<I", len(tris)))
        f.write(rec.tobytes())


class GMesh(GPrim):
    """Triangle-mesh geometry (mcramp/geom/mesh.py:34-98, mesh.cl:3-129).

    The reference tests every triangle for every ray (Moller-Trumbore, eps
    1e-9): the earliest entering face gives intersection 1, the earliest
    exiting face intersection 2, and ``interior`` uses the crossing-count
    parity.  The CUDA kernel returns the same records through a bounding
    volume hierarchy built at plan creation.
    Slots: gp[0..5] = x_min, x_max, y_min, y_max, z_min, z_max (float32
    bounds of the vertices), gi[0] = interior, table[0] = points [n_tri*9]."""
    kind = _abi.G_MESH

    def __init__(self, filename='', interior=False, idx=0, ctx=None, points=None):
        self.idx = np.uint32(idx)
        self.filename = filename
        self.points = read_stl_cached(filename) if points is None else \
            np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 9)
        allv = self.points.reshape(-1, 3)
        mn, mx = allv.min(axis=0), allv.max(axis=0)
        (self.x_min, self.y_min, self.z_min) = (np.float32(v) for v in mn)
        (self.x_max, self.y_max, self.z_max) = (np.float32(v) for v in mx)
        self.num_tri = np.uint32(len(self.points))
        self.interior = np.uint32(1 if interior else 0)

    def fill(self, comp, keep):
        super().fill(comp, keep)
        for k, v in enumerate((self.x_min, self.x_max, self.y_min, self.y_max,
                               self.z_min, self.z_max)):
            comp.gp[k] = v
        comp.gi[0] = int(self.interior)
        _abi.set_table(comp, 0, self.points, keep)
