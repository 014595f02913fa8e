"""The host BVH builder (ramp_gb300/csrc/bvh.cpp) and the node layout the
GMesh walk reads (ramp_gb300/csrc/mesh.cuh): every triangle sits in exactly
one leaf, and a walk that follows the layout's rules (test both children of
an inner node, take the triangles of leaf children, go on into inner
children) reaches every triangle that a ray hits by the reference's
Moller-Trumbore test (mesh.cl:42-111), checked by brute force in float32.
The builder is compiled here with g++ behind a small C shim."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "ramp_gb300", "csrc")
SHIM = r'''
#include <cstring>
#include <vector>
#include "bvh.h"
extern "C" int bvh_build(const float* pts, long long n_tri, float* nodes, long long* n_nodes,
                         float* tris) {
  std::vector<float> nd, tr;
  int rc = ramp_bvh_build(pts, n_tri, nd, tr);
  if (rc) return rc;
  if ((long long)nd.size() > *n_nodes) return -2;
  std::memcpy(nodes, nd.data(), nd.size() * 4);
  std::memcpy(tris, tr.data(), tr.size() * 4);
  *n_nodes = (long long)nd.size();
  return 0;
}
'''


@pytest.fixture(scope="module")
def builder(tmp_path_factory):
    d = tmp_path_factory.mktemp("bvh")
    src = d / "shim.cpp"
    src.write_text(SHIM)
    so = d / "libbvh.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC,
                           str(src), os.path.join(CSRC, "bvh.cpp"), "-o", str(so)])
    lib = ctypes.CDLL(str(so))
    lib.bvh_build.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p]
    lib.bvh_build.restype = ctypes.c_int

    def build(tris):
        n = len(tris)
        cap = np.array([16 * max(2 * n, 1)], dtype=np.int64)
        nodes = np.zeros(int(cap[0]), np.float32)
        out = np.zeros(12 * n, np.float32)
        assert lib.bvh_build(tris.ctypes.data, n, nodes.ctypes.data, cap.ctypes.data,
                             out.ctypes.data) == 0
        return nodes[:int(cap[0])].reshape(-1, 16), out.reshape(-1, 12)
    return build


def torus(rng, nu, nv, R=0.05, r=0.02, noise=0.002):
    u = np.linspace(0, 2 * np.pi, nu, endpoint=False)
    v = np.linspace(0, 2 * np.pi, nv, endpoint=False)
    U, V = np.meshgrid(u, v, indexing="ij")
    rr = r + noise * rng.standard_normal(U.shape)
    P = np.stack([(R + rr * np.cos(V)) * np.cos(U), rr * np.sin(V),
                  (R + rr * np.cos(V)) * np.sin(U)], -1)
    a = P
    b = np.roll(P, -1, axis=0)
    c = np.roll(b, -1, axis=1)
    d = np.roll(P, -1, axis=1)
    t1 = np.concatenate([a, b, c], -1).reshape(-1, 9)
    t2 = np.concatenate([a, c, d], -1).reshape(-1, 9)
    return np.ascontiguousarray(np.concatenate([t1, t2]), dtype=np.float32)


def leaves_reached(nodes, pos, vel):
    """Triangles in the leaves a walk reaches (the rules of mesh_step)."""
    ni = nodes.view(np.int32)
    with np.errstate(divide="ignore"):
        inv = (np.float32(1) / vel).astype(np.float32)
    reached = []
    stack, node = [], 0
    while True:
        inner = []
        for c in (0, 8):
            b = ni[node, c + 7]
            if b < 0:
                continue
            lo, hi = nodes[node, c:c + 3], nodes[node, c + 4:c + 7]
            with np.errstate(invalid="ignore"):
                t0, t1 = (lo - pos) * inv, (hi - pos) * inv
            tn, tf = np.max(np.minimum(t0, t1)), np.min(np.maximum(t0, t1))
            if tn > tf or tf < -1e-6:
                continue
            if b >= 1:
                reached.append((ni[node, c + 3], b))
            else:
                inner.append(ni[node, c + 3])
        if len(inner) == 2:
            stack.append(inner[1])
            node = inner[0]
        elif inner:
            node = inner[0]
        elif stack:
            node = stack.pop()
        else:
            return reached


def mt_hits(tris, pos, vel):
    v0, v1, v2 = tris[:, 0:3], tris[:, 4:7], tris[:, 8:11]
    e1, e2 = v1 - v0, v2 - v0
    h = np.cross(vel, e2)
    aa = np.einsum("ij,ij->i", e1, h)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.float32(1) / aa
        sv = pos - v0
        u = f * np.einsum("ij,ij->i", sv, h)
        qv = np.cross(sv, e1)
        v = f * (qv @ vel)
        t = f * np.einsum("ij,ij->i", e2, qv)
        return (np.abs(aa) >= 1e-9) & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1) & (t > 1e-9)


@pytest.mark.parametrize("nu,nv,keep", [(40, 20, 3), (40, 20, None), (120, 60, None)])
def test_leaves_partition_the_triangles_and_walks_reach_every_hit(builder, nu, nv, keep):
    """keep = 3: a mesh small enough that the root is a leaf (one node with
    one child)."""
    rng = np.random.default_rng(nu * 1000 + nv)
    pts = torus(rng, nu, nv)
    if keep:
        pts = np.ascontiguousarray(pts[:keep])
    nodes, tris = builder(pts)
    if keep:
        assert len(nodes) == 1 and nodes.view(np.int32)[0, 15] == -1
    ni = nodes.view(np.int32)
    seen = np.zeros(len(tris), int)
    for c in (0, 8):
        for a, b in zip(ni[:, c + 3], ni[:, c + 7]):
            if b >= 1:
                seen[a:a + b] += 1
    assert (seen == 1).all()
    # sibling leaves hold adjacent triangle ranges: a walk that takes both
    # leaf children of a node tests one range [a0, a1 + b1)
    both = (ni[:, 7] >= 1) & (ni[:, 15] >= 1)
    assert (ni[both, 11] == ni[both, 3] + ni[both, 7]).all()
    hits_total = 0
    for _ in range(150):
        pos = rng.uniform(-0.1, 0.1, 3).astype(np.float32)
        pos[2] = -0.5
        tgt = rng.uniform(-0.08, 0.08, 3).astype(np.float32)
        tgt[2] = 0.0
        vel = ((tgt - pos) * np.float32(300.0)).astype(np.float32)
        mask = np.zeros(len(tris), bool)
        for a, b in leaves_reached(nodes, pos, vel):
            mask[a:a + b] = True
        hit = mt_hits(tris, pos, vel)
        hits_total += int(hit.sum())
        assert not (hit & ~mask).any()
    assert keep or hits_total > 0


def walk_counts(nodes, pos, vel):
    """(inner nodes read, triangles read) of the walk by the rules above."""
    ni = nodes.view(np.int32)
    with np.errstate(divide="ignore"):
        inv = (np.float32(1) / vel).astype(np.float32)
    n_nodes, n_tris, stack = 0, 0, [0]
    while stack:
        node = stack.pop()
        n_nodes += 1
        for c in (0, 8):
            b = ni[node, c + 7]
            if b < 0:
                continue
            lo, hi = nodes[node, c:c + 3], nodes[node, c + 4:c + 7]
            with np.errstate(invalid="ignore"):
                t0, t1 = (lo - pos) * inv, (hi - pos) * inv
            tn, tf = np.max(np.minimum(t0, t1)), np.min(np.maximum(t0, t1))
            if tn > tf or tf < -1e-6:
                continue
            if b >= 1:
                n_tris += int(b)
            else:
                stack.append(ni[node, c + 3])
    return n_nodes, n_tris


def test_library_walk_counts_match_the_layout_walk(builder):
    """ramp_bvh_walk_counts (the mesh roofline's algorithmic L2 bytes) reads
    the hierarchy the library builds as the layout walk does; a ray that
    misses the mesh's box reads nothing."""
    import ctypes
    from ramp_gb300 import _abi
    lib = _abi.load()
    rng = np.random.default_rng(9)
    pts = torus(rng, 60, 30)
    nodes, _ = builder(pts)
    rays = []
    for _ in range(120):
        pos = rng.uniform(-0.1, 0.1, 3).astype(np.float32)
        pos[2] = -0.5
        tgt = rng.uniform(-0.08, 0.08, 3).astype(np.float32)
        tgt[2] = 0.0
        rays.append(np.concatenate([pos, (tgt - pos) * np.float32(300.0)]))
    rays.append(np.array([5.0, 5.0, -0.5, 0.0, 0.0, 300.0], np.float32))   # misses the box
    rays = np.ascontiguousarray(np.array(rays, np.float32))
    lo, hi = pts.reshape(-1, 3).min(0), pts.reshape(-1, 3).max(0)
    want = np.zeros(3, np.int64)
    for r in rays:
        pos, vel = r[:3], r[3:]
        with np.errstate(divide="ignore", invalid="ignore"):
            t1, t2 = (lo - pos) / vel, (hi - pos) / vel
        if np.min(np.maximum(t1, t2)) < 0 or np.max(np.minimum(t1, t2)) > np.min(np.maximum(t1, t2)):
            continue
        a, b = walk_counts(nodes, pos, vel)
        want += (a, b, 1)
    out = np.zeros(3, np.int64)
    assert lib.ramp_bvh_walk_counts(pts.ctypes.data, len(pts), rays.ctypes.data, len(rays),
                                    out.ctypes.data) == 0
    assert 10 < want[2] < len(rays)
    assert np.array_equal(out, want)
