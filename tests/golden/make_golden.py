"""Generate tests/golden/ref_pins.npz from the reference's own code.

Runs in a checkout where the reference is present: it builds
oracle/_ref/libref_pins.so from the reference's mcramp/include/rand.h (with
its vendored Random123 headers) and mcramp/include/ref.h, unmodified, and
records:
  threefry_ctr0, threefry_tid, threefry_x   Threefry-4x32-20 word x for the
                                            reference key/counter layout
  rand_tid, rand_sb0, rand_u, rand_sb       64 successive rand() draws per
                                            (tid, initial sb) and the
                                            counter after each draw
  refl_params, refl_q, refl_R               reflectivity_func samples
The GPU machine has no reference checkout; the tests read these fixtures there.

    python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402

REFL_PARAMS = np.array([[0.99, 0.0219, 3.0, 2.0, 0.003],     # LET-like guides
                        [1.0, 0.0218, 4.38, 4.0, 0.003],     # examples/LET.json
                        [0.99, 0.0219, 0.0, 2.0, 0.0],       # m-parametrisation
                        [0.99, 0.0219, 0.0, 4.0, 0.0],
                        [0.9, 0.0219, 2.0, 0.5, 0.002],      # m < 1
                        [0.0, 0.0219, 3.0, 2.0, 0.003],      # R0 = 0
                        [0.99, 0.0219, 3.0, 2.0, 0.0]],      # W = 0, alpha != 0
                       dtype=np.float32)


def main():
    P = oracle.pins()
    if P is None:
        raise SystemExit("reference checkout not found; set RAMP_REFERENCE")
    rng = np.random.default_rng(20261203)
    n = 4096
    ctr0 = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    tid = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    ctr0[:8] = [0, 1, 2, 3, 4096, 4097, 0xffffffff, 0x7fffffff]
    tid[:8] = [0, 0, 0, 0, 1, 2, 0xffffffff, 12345]
    x = np.zeros(n, np.uint32)
    P.ref_pin_threefry(ctr0.ctypes.data, tid.ctypes.data, x.ctypes.data, n)

    tids = np.array([0, 1, 2, 31, 1000, 999999, 123456789], np.uint32)
    sb0s = np.array([0.0, 1.0, 17.0, 4096.0, 8191.0, 100000.0], np.float32)
    rt, rs, ru, rsb = [], [], [], []
    for t in tids:
        for sb0 in sb0s:
            rec = np.zeros(16, np.float32)
            rec[11] = sb0
            us, sbs = [], []
            for _ in range(64):
                us.append(P.ref_pin_rand(rec.ctypes.data, int(t)))
                sbs.append(rec[11])
            rt.append(t); rs.append(sb0); ru.append(us); rsb.append(sbs)

    q = np.concatenate([np.linspace(0.0, 0.2, 2001), [0.0219, 0.0438, 0.0876]]).astype(np.float32)
    R = np.zeros((len(REFL_PARAMS), len(q)), np.float32)
    for i, prm in enumerate(REFL_PARAMS):
        for j, qq in enumerate(q):
            R[i, j] = P.ref_pin_reflectivity(float(qq), *[float(v) for v in prm])
    out = os.path.join(HERE, "ref_pins.npz")
    np.savez_compressed(out, threefry_ctr0=ctr0, threefry_tid=tid, threefry_x=x,
                        rand_tid=np.array(rt, np.uint32), rand_sb0=np.array(rs, np.float32),
                        rand_u=np.array(ru, np.float32), rand_sb=np.array(rsb, np.float32),
                        refl_params=REFL_PARAMS, refl_q=q, refl_R=R)
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
