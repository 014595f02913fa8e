"""ramp_trace_batched_noalloc: the batched fused path for callers that may
not allocate device memory while tracing.  Its scratch lives in a fixed
device array inside the library; its results must equal those of
ramp_trace_batched (the allocating entry point) on the same inputs, call
after call, up to the order of float atomic additions in the tallies.

Kept in a file of its own, collected last, and self-contained, so that it
runs the same alone in a fresh process and after the other GPU tests.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

import ramp_gb300 as m
from ramp_gb300 import _abi, instruments as I

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24
GOLD_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def assert_tallies_match(a_inst, b_inst):
    """Per bin |a - b| <= 2 (n_eff + 1) u |b| + 1e-12 max|b|, n_eff = H^2/E."""
    ta, tb = a_inst.tallies(), b_inst.tallies()
    for k in range(0, len(tb), 2):
        H = tb[k].cpu().double().numpy()
        E = tb[k + 1].cpu().double().numpy()
        n_eff = np.where(E > 0, H * H / np.where(E > 0, E, 1.0), 1.0)
        for j in (k, k + 1):
            x = ta[j].cpu().double().numpy()
            y = tb[j].cpu().double().numpy()
            tol = 2 * (n_eff + 1) * U32 * np.abs(y) + 1e-12 * max(np.abs(y).max(), 1e-30)
            assert (np.abs(x - y) <= tol).all(), "tally %d differs" % j
            assert np.array_equal(x != 0, y != 0)


def variants_of(insts, counts, seeds):
    keep = []
    arr = (_abi.RampVariant * len(insts))()
    for v, (inst, n, seed) in enumerate(zip(insts, counts, seeds)):
        src, carr, nc, barr, nb = inst.descriptors(keep)
        keep.append(carr)
        arr[v].comps = ctypes.cast(carr, ctypes.POINTER(_abi.RampComp))
        arr[v].source = src
        arr[v].n = n
        arr[v].num_sim = n
        arr[v].seed = seed
    return arr, keep


def test_noalloc_batched_equals_allocating_entry_point(cuda_lib):
    lib = cuda_lib
    kws = [I.let_like_kwargs(Ei=3.7, use_slit=1, slit_w=0.03),
           I.let_like_kwargs(Ei=7.5, use_slit=1, slit_w=0.012),
           I.let_like_kwargs(Ei=2.2, use_slit=1, slit_w=0.04)]
    counts = [400_000, 150_001, 250_003]
    seeds = [101, 2048, 4095]
    fn = I.path("let_like.json")
    A = [m.Instrument(fn, "cuda", **kw) for kw in kws]      # ramp_trace_batched
    B = [m.Instrument(fn, "cuda", **kw) for kw in kws]      # ramp_trace_batched_noalloc
    plan_a, plan_b = A[0].plan(), B[0].plan()
    va, keep_a = variants_of(A, counts, seeds)
    vb, keep_b = variants_of(B, counts, seeds)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for mode in (1, 0, 1):           # native, reference, native again: three calls in a row
        rng = _abi.RampRng(mode, 77, 0, 0)
        _abi.check(lib, lib.ramp_trace_batched(plan_a, va, len(A), ctypes.byref(rng), None,
                                               stream), "ramp_trace_batched")
        _abi.check(lib, lib.ramp_trace_batched_noalloc(plan_b, vb, len(B), ctypes.byref(rng),
                                                       None, stream),
                   "ramp_trace_batched_noalloc")
        torch.cuda.synchronize()
        assert sum(float(t.sum()) for b in B for t in b.tallies()) > 0
        for a, b in zip(A, B):
            assert_tallies_match(a, b)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    lib = cuda_lib
    inst = m.Instrument(I.path("let_like.json"), "cuda", **I.let_like_kwargs())
    plan = inst.plan()
    arr, keep = variants_of([inst] * 257, [1000] * 257, [1] * 257)
    rng = _abi.RampRng(1, 0, 0, 0)
    rc = lib.ramp_trace_batched_noalloc(plan, arr, 257, ctypes.byref(rng), None, None)
    assert rc == -6
    assert "exceed the fixed scratch" in _abi.last_error(lib)


def plan_status(lib, plan):
    flags, oob = ctypes.c_uint32(), ctypes.c_uint64()
    _abi.check(lib, lib.ramp_plan_status(plan, ctypes.byref(flags), ctypes.byref(oob)),
               "ramp_plan_status")
    return flags.value, oob.value


def test_noalloc_reports_device_status_through_the_plan(cuda_lib):
    """A chain whose monitors drop out-of-range tally writes: the drops
    counted by the no-allocation entry point reach ramp_plan_status, as
    those of the allocating entry point do, on two calls in a row."""
    lib = cuda_lib
    fn = os.path.join(GOLD_DIR, "guides_monitors.json")
    kw = I.small_chain_kwargs()
    A = m.Instrument(fn, "cuda", **kw)
    B = m.Instrument(fn, "cuda", **kw)
    plan_a, plan_b = A.plan(), B.plan()
    va, keep_a = variants_of([A, A], [100_000, 60_001], [5, 9])
    vb, keep_b = variants_of([B, B], [100_000, 60_001], [5, 9])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    plan_status(lib, plan_a)
    plan_status(lib, plan_b)
    for _ in range(2):
        rng = _abi.RampRng(0, 0, 0, 0)
        _abi.check(lib, lib.ramp_trace_batched(plan_a, va, 2, ctypes.byref(rng), None, stream),
                   "ramp_trace_batched")
        _abi.check(lib, lib.ramp_trace_batched_noalloc(plan_b, vb, 2, ctypes.byref(rng), None,
                                                       stream), "ramp_trace_batched_noalloc")
        fa, oa = plan_status(lib, plan_a)
        fb, ob = plan_status(lib, plan_b)
        assert oa > 0
        assert (fb, ob) == (fa, oa)
        assert fb & _abi.F_WORKQ == 0
    assert_tallies_match(A, B)


@pytest.mark.parametrize("fn,kws,counts,seeds", [
    ("mesh_imaging.json", [I.mesh_imaging_kwargs(angle=0.0), I.mesh_imaging_kwargs(angle=0.9)],
     [30_000, 20_011], [7, 8]),
    ("let_like_misis.json", [I.let_like_misis_kwargs(Ei=3.7), I.let_like_misis_kwargs(Ei=6.0)],
     [200_000, 90_001], [3, 4000])])
def test_noalloc_mesh_and_extended_kinds_equal_allocating_entry_point(cuda_lib, fn, kws,
                                                                      counts, seeds):
    """Descriptors that point at tables the plan already holds (a mesh's
    hierarchy, the MISIS spectrum tables) are looked up, not uploaded, and
    trace as the allocating entry point does, on two calls in a row."""
    lib = cuda_lib
    A = [m.Instrument(I.path(fn), "cuda", **kw) for kw in kws]
    B = [m.Instrument(I.path(fn), "cuda", **kw) for kw in kws]
    plan_a, plan_b = A[0].plan(), B[0].plan()
    va, keep_a = variants_of(A, counts, seeds)
    vb, keep_b = variants_of(B, counts, seeds)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for mode in (0, 1):
        rng = _abi.RampRng(mode, 5, 0, 0)
        _abi.check(lib, lib.ramp_trace_batched(plan_a, va, len(A), ctypes.byref(rng), None,
                                               stream), "ramp_trace_batched")
        _abi.check(lib, lib.ramp_trace_batched_noalloc(plan_b, vb, len(B), ctypes.byref(rng),
                                                       None, stream),
                   "ramp_trace_batched_noalloc")
        torch.cuda.synchronize()
        for a, b in zip(A, B):
            assert_tallies_match(a, b)
    assert sum(float(t.sum()) for b in B for t in b.tallies()) > 0
