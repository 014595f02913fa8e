"""Differentiable detector histograms.

No reference counterpart: RAMP has no gradients.  ``DiffChain`` exposes a
set of parameters that enter neutron weights smoothly — supermirror guide
R0, Qc, alpha, m, W (reflectivity per bounce, mcramp/include/ref.h), the
moderator temperature (MCont, cont_mod.cl:4-9; T1 = T2 = T3) and the powder
absorption cross-section (SPowderN sigma_abs, powderN.cl:31-33,55,118) —
and one histogram detector.  ``forward`` runs the fused path with explicit
chunk parameters (common random numbers across calls); ``gradient`` runs
the adjoint kernel (ramp_adjoint) for dL/dH of that detector.
``histogram(chain, theta, n, seed)`` wraps both in a torch.autograd.Function,
so a loss written in torch differentiates end to end:

    chain = DiffChain(inst, [("guide1", "R0"), ..., ("mod", "T"),
                             ("sample", "sigma_abs")], detector="detector")
    theta = chain.values().requires_grad_()
    H = histogram(chain, theta, 10_000_000, seed=1)
    loss = ((H.double() - H_target) ** 2).sum()
    loss.backward()            # theta.grad from the adjoint kernel

The default estimator is pathwise (the powder penetration depth
reparameterised through its inverse CDF, every branch held fixed): the
derivative that central finite differences with common random numbers
measure.  ``lr=True`` adds the likelihood-ratio score of the powder's
transmit/scatter branch, which makes the estimator unbiased for the
expected histogram.
"""
import ctypes

import numpy as np
import torch

from . import _abi

GUIDE_KINDS = {"R0": _abi.DP_GUIDE_R0, "Qc": _abi.DP_GUIDE_QC, "alpha": _abi.DP_GUIDE_ALPHA,
               "m": _abi.DP_GUIDE_M, "W": _abi.DP_GUIDE_W}


class DiffChain:
    def __init__(self, inst, params, detector):
        self.inst = inst
        comps = inst.components()
        names = [name for name, _ in comps]
        self.spec = []            # (kind, comp index, scale to descriptor value)
        self.names = []
        for comp_name, attr in params:
            if attr == "T":
                src = inst.source
                if not hasattr(src, "T1"):
                    raise ValueError("the source has no temperature")
                self.spec.append((_abi.DP_SOURCE_T, -1, 1.0, src))
            else:
                j = names.index(comp_name)
                scat = comps[j][1]["scat_kernel"]
                if attr in GUIDE_KINDS:
                    if scat.kind != _abi.S_GUIDE:
                        raise ValueError("%s is not a guide" % comp_name)
                    self.spec.append((GUIDE_KINDS[attr], j, 1.0, scat))
                elif attr == "sigma_abs":
                    if scat.kind != _abi.S_POWDERN:
                        raise ValueError("%s is not a powder" % comp_name)
                    # descriptor value sigma_abs*v = pack * sigma_abs / vc * 100
                    self.spec.append((_abi.DP_POWDER_SIGMA_ABS, j, scat.pack / scat.vc * 100.0,
                                      scat))
                else:
                    raise ValueError("no differentiable parameter %r" % attr)
            self.names.append("%s.%s" % (comp_name, attr))
        self.det = names.index(detector)
        self.det_scat = comps[self.det][1]["scat_kernel"]
        self.params = (_abi.RampDiffParam * len(self.spec))(
            *[_abi.RampDiffParam(k, max(j, 0)) for k, j, _, _ in self.spec])
        self._theta = self.values().tolist()

    def values(self):
        """Current parameter values (guide attributes, T1, sigma_abs)."""
        out = []
        for (kind, j, scale, obj), name in zip(self.spec, self.names):
            attr = name.split(".")[-1]
            if kind == _abi.DP_SOURCE_T:
                out.append(float(obj.T1))
            elif kind == _abi.DP_POWDER_SIGMA_ABS:
                out.append(float(obj.sigma_abs))
            else:
                out.append(float(getattr(obj, attr)))
        return torch.tensor(out, dtype=torch.float64)

    def set(self, theta):
        lib = self.inst._lib()
        plan = self.inst.plan()
        theta = [float(t) for t in (theta.tolist() if torch.is_tensor(theta) else theta)]
        for (kind, j, scale, obj), v in zip(self.spec, theta):
            _abi.check(lib, lib.ramp_plan_set_param(plan, kind, j, float(np.float32(v * scale))),
                       "ramp_plan_set_param")
        self._theta = theta
        self.inst._param_epoch = getattr(self.inst, "_param_epoch", 0) + 1

    def forward(self, n, seed, rng="reference"):
        """The detector histogram (flat, float32, device) of n histories at
        the current parameters, one chunk with weight 1/n and this seed.
        The run also lists the neutrons the detector counts, which the
        next ``gradient`` of the same run replays (ramp_forward_record)."""
        lib = self.inst._lib()
        plan = self.inst.plan()
        self.inst.reset_tallies()
        rngd = _abi.RampRng({"reference": 0, "native": 1}[rng], 0, 0, 0, None)
        with torch.cuda.device(self.inst.device):
            stream = self.inst._stream_ptr()
            _abi.check(lib, lib.ramp_forward_record(plan, self.det, int(n), int(n), int(seed),
                                                    ctypes.byref(rngd), stream),
                       "ramp_forward_record")
        return self.det_scat.tallies()[0]

    def gradient(self, dLdH, n, seed, rng="reference", lr=False):
        """dL/dtheta (float64, len(params)) for dL/dH of the detector."""
        lib = self.inst._lib()
        plan = self.inst.plan()
        g = dLdH.detach().to(device=self.inst.device, dtype=torch.float32).contiguous().view(-1)
        if g.numel() != self.det_scat.tallies()[0].numel():
            raise ValueError("dL/dH has the wrong size for the detector")
        grad = torch.zeros(len(self.spec), dtype=torch.float64, device=self.inst.device)
        rngd = _abi.RampRng({"reference": 0, "native": 1}[rng], 0, 0, 0)
        with torch.cuda.device(self.inst.device):
            stream = self.inst._stream_ptr()
            _abi.check(lib, lib.ramp_adjoint(plan, self.params, len(self.spec), self.det,
                                             ctypes.c_void_p(g.data_ptr()), int(n), int(n),
                                             int(seed), ctypes.byref(rngd), 1 if lr else 0,
                                             ctypes.c_void_p(grad.data_ptr()), stream),
                       "ramp_adjoint")
        scale = torch.tensor([s for _, _, s, _ in self.spec], dtype=torch.float64,
                             device=grad.device)
        return grad * scale


class _Histogram(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, chain, n, seed, rng, lr):
        chain.set(theta.detach().cpu())
        H = chain.forward(n, seed, rng).clone()
        ctx.chain, ctx.n, ctx.seed, ctx.rng, ctx.lr = chain, n, seed, rng, lr
        ctx.theta = theta.detach().cpu().clone()
        ctx.theta_dtype, ctx.theta_device = theta.dtype, theta.device
        return H

    @staticmethod
    def backward(ctx, gH):
        chain = ctx.chain
        chain.set(ctx.theta)
        g = chain.gradient(gH, ctx.n, ctx.seed, ctx.rng, ctx.lr)
        return g.to(dtype=ctx.theta_dtype, device=ctx.theta_device), None, None, None, None, None


def histogram(chain, theta, n, seed, rng="reference", lr=False):
    """Detector histogram as a differentiable function of theta."""
    return _Histogram.apply(theta, chain, int(n), int(seed), rng, bool(lr))


LET_LIKE_PARAMS = ([("guide%d" % g, a) for g in (1, 2, 3, 4) for a in ("R0", "Qc", "alpha", "m", "W")]
                   + [("mod", "T"), ("sample", "sigma_abs")])
