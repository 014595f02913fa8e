"""Comparison helpers shared by the parity tests.

Per-neutron records must be bit-identical (NaN equal to NaN).  Histograms
may differ only by the order of float additions: for a bin holding
H = sum(p) with E = sum(p^2), n_eff = H^2/E terms; recursive float summation
of positive terms errs by at most (n-1) u H on each side (u = 2^-24), so per
bin |a - b| <= 2 (n_eff + 1) u |H| + 1e-12 max|H|.
"""
import numpy as np


def records_equal(a, b):
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    if not eq.all():
        bad = np.argwhere(~eq)
        i, l = bad[0]
        raise AssertionError("%d mismatching values; first at neutron %d lane %d: gpu %r cpu %r\n"
                             "gpu %r\ncpu %r" % (len(bad), i, l, a[i, l], b[i, l], a[i], b[i]))


U32 = 2.0 ** -24


def tallies_close(g_inst, c_inst):
    tg_all, tc_all = g_inst.tallies(), c_inst.tallies()
    for k, (tg, tc) in enumerate(zip(tg_all, tc_all)):
        g = tg.cpu().numpy().astype(np.float64)
        c = tc.numpy().astype(np.float64)
        # n_eff from the (sum p, sum p^2) pair this tally belongs to
        if k % 2 == 0 and k + 1 < len(tc_all) and tc_all[k + 1].numel() == tc.numel():
            H, E = c, tc_all[k + 1].numpy().astype(np.float64)
        elif k % 2 == 1 and tc_all[k - 1].numel() == tc.numel():
            H, E = tc_all[k - 1].numpy().astype(np.float64), c
        else:
            H, E = c, None
        n_eff = np.where(E > 0, H * H / np.where(E > 0, E, 1), 1.0) if E is not None else \
            np.full_like(c, 1e6)
        tol = 2 * (n_eff + 1) * U32 * np.abs(c) + 1e-12 * max(np.abs(c).max(), 1e-30)
        bad = np.abs(g - c) > tol
        assert not bad.any(), "tally %d: %d bins differ, worst %g vs tol %g" % (
            k, bad.sum(), np.abs(g - c)[bad].max(), tol[bad][np.argmax(np.abs(g - c)[bad])])
        assert np.array_equal(g != 0, c != 0)


class _Host:
    """Host view of another instrument's tallies (for GPU-vs-GPU checks)."""
    def __init__(self, inst):
        self._t = [t.cpu() for t in inst.tallies()]

    def tallies(self):
        return self._t


