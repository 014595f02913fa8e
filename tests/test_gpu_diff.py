"""Gradients of a detector-histogram loss from the adjoint kernel against
central finite differences with common random numbers.

LET-like chain at 1e7 histories; 22 parameters: 4 guides x (R0, Qc, alpha,
m, W), the moderator temperature and the powder sigma_abs.  The target
histogram is the chain at theta0 * (1 + 0.05 N(0,1)) (numpy seed 23, another
RNG seed); loss = sum (H - H_target)^2.  Central differences use a relative
step of 1e-3 and the same seed on both sides.  Agreement: 2 % of each
component (a floor of 1e-6 of the largest component only guards a
component that is exactly zero).
"""
import numpy as np
import pytest
import torch

import ramp_gb300 as m
from ramp_gb300 import instruments as I
from ramp_gb300.diff import DiffChain, LET_LIKE_PARAMS, histogram

pytestmark = pytest.mark.gpu

N = 10_000_000


@pytest.fixture(scope="module")
def problem(cuda_lib):
    inst = m.Instrument(I.path("let_like.json"), "cuda", **I.let_like_kwargs())
    chain = DiffChain(inst, LET_LIKE_PARAMS, detector="detector")
    theta0 = chain.values()
    r = np.random.default_rng(23)
    theta_t = theta0 * (1.0 + 0.05 * torch.tensor(r.standard_normal(len(theta0))))
    chain.set(theta_t)
    Ht = chain.forward(N, seed=999).double().clone()
    chain.set(theta0)
    return chain, theta0, Ht


def loss(chain, theta, seed, Ht, lr=False):
    H = histogram(chain, theta, N, seed, lr=lr)
    return ((H.double() - Ht) ** 2).sum()


def adjoint_grad(chain, theta0, Ht, seed=1, lr=False):
    th = theta0.clone().requires_grad_()
    L = loss(chain, th, seed, Ht, lr)
    L.backward()
    return th.grad.clone(), float(L.detach())


def test_adjoint_matches_central_differences(problem):
    chain, theta0, Ht = problem
    g, L0 = adjoint_grad(chain, theta0, Ht)
    assert L0 > 0
    fd = torch.zeros_like(g)
    with torch.no_grad():
        for k in range(len(theta0)):
            h = 1e-3 * float(theta0[k])
            tp, tm = theta0.clone(), theta0.clone()
            tp[k] += h
            tm[k] -= h
            fd[k] = (loss(chain, tp, 1, Ht) - loss(chain, tm, 1, Ht)) / (2 * h)
    scale = float(fd.abs().max())
    assert scale > 0
    bad = (g - fd).abs() > 0.02 * fd.abs() + 1e-6 * scale
    assert not bad.any(), "\n".join(
        "%-16s adjoint %+.6e  fd %+.6e" % (chain.names[k], g[k], fd[k]) for k in range(len(g)))


def test_likelihood_ratio_terms_only_touch_branching_parameters(problem):
    """The likelihood-ratio estimator adds the score of the powder's
    transmit/scatter choice: only the absorption gradient changes."""
    chain, theta0, Ht = problem
    g0, _ = adjoint_grad(chain, theta0, Ht, seed=5)
    g1, _ = adjoint_grad(chain, theta0, Ht, seed=5, lr=True)
    k = chain.names.index("sample.sigma_abs")
    others = [j for j in range(len(g0)) if j != k]
    # the same per-neutron terms against a forward histogram (hence dL/dH)
    # that differs only by the order of its float additions
    d = (g0[others] - g1[others]).abs()
    tol = 1e-5 * g0[others].abs() + 1e-6 * float(g0.abs().max())
    assert bool((d <= tol).all()), "max |diff| %g" % float(d.max())
    assert abs(float(g1[k] - g0[k])) > 1e-3 * abs(float(g0[k]))


def test_adjoint_is_deterministic_in_value(problem):
    chain, theta0, Ht = problem
    a, _ = adjoint_grad(chain, theta0, Ht, seed=3)
    b, _ = adjoint_grad(chain, theta0, Ht, seed=3)
    assert torch.allclose(a, b, rtol=1e-6, atol=1e-3 * float(a.abs().max()))


def test_likelihood_ratio_pathwise_and_finite_differences_agree_statistically(cuda_lib):
    """The three estimators over 16 seeds of 1e7 histories, for the linear
    loss L = sum of the detector histogram (its gradient is dE[H]/dtheta
    summed over bins, so per-seed estimates average to the derivative).

    * The moderator temperature and guide 1's m enter only weights: the
      pathwise estimate is the likelihood-ratio one (no branch depends on
      them) and both equal central differences with common random numbers
      at step 1e-3 to 1e-3 of the mean.
    * sample.sigma_abs also moves the powder's transmit/scatter threshold:
      finite differences see that only through neutrons that change branch,
      which a step of 5e-2 samples; there the likelihood-ratio estimate
      (pathwise plus the score of the branch) agrees with them within three
      standard errors of the paired differences, closer than the pathwise
      estimate, which leaves the branch out."""
    inst = m.Instrument(I.path("let_like.json"), "cuda", **I.let_like_kwargs())
    chain = DiffChain(inst, [("sample", "sigma_abs"), ("mod", "T"), ("guide1", "m")],
                      detector="detector")
    theta0 = chain.values()
    L = lambda H: H.double().sum()
    path, lr, fd = [], [], []
    steps = (5e-2, 1e-3, 1e-3)
    for seed in range(300, 316):
        for estimates, use_lr in ((path, False), (lr, True)):
            th = theta0.clone().requires_grad_()
            L(histogram(chain, th, N, seed, lr=use_lr)).backward()
            estimates.append(th.grad.clone().numpy())
        row = []
        with torch.no_grad():
            for k, rel in enumerate(steps):
                h = rel * float(theta0[k])
                tp, tm = theta0.clone(), theta0.clone()
                tp[k] += h
                tm[k] -= h
                row.append(float((L(histogram(chain, tp, N, seed)) -
                                  L(histogram(chain, tm, N, seed))) / (2 * h)))
        fd.append(row)
    path, lr, fd = np.array(path), np.array(lr), np.array(fd)
    for k in (1, 2):                       # weights only: one estimator (up to the
        assert np.allclose(path[:, k], lr[:, k], rtol=1e-9, atol=0)   # order of additions)
        assert abs(path[:, k].mean() - fd[:, k].mean()) <= 1e-3 * abs(fd[:, k].mean())
    d = lr[:, 0] - fd[:, 0]
    se = d.std(ddof=1) / np.sqrt(len(d))
    assert abs(d.mean()) <= 3 * se, (lr[:, 0].mean(), fd[:, 0].mean(), se)
    assert abs(d.mean()) < abs((path[:, 0] - fd[:, 0]).mean())
