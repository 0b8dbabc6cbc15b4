"""Q1 adjoint on the GPU: dJ/d log a against central finite differences of the
GPU forward, against the plain FP64 path's gradient, the oracle's gradient, and
through torch.autograd.

Finite differences: h = 1e-6, forward solves at rtol 1e-14; stated tolerance
|FD - grad.d| <= 1e-6 * sum_i |grad_i d_i| (the directional derivative's scale
without cancellation), and <= 1e-6 relative to |FD| wherever the directional
derivative is not cancelled (|FD| >= 0.1 sum_i |grad_i d_i|)."""
import numpy as np
import pytest

import workloads
from adjoint_harness import MisfitProblem, make_autograd

pytestmark = pytest.mark.gpu


def _problem(gpu, precision, m=2, depth=3, npts=40, seed=11, rtol=None):
    cells, a, r, load = workloads.q1_lognormal(m=m, depth=depth, seed=seed, reaction=False)
    rng = np.random.default_rng(seed + 1)
    cell_of = rng.integers(0, len(cells), npts)
    pts = cells["origin"][cell_of] + rng.random((npts, 3)) * cells["size"][cell_of]
    # data from a second seeded coefficient
    _, a2, _, _ = workloads.q1_lognormal(m=m, depth=depth, seed=seed + 2, reaction=False)
    p2 = MisfitProblem(gpu, cells, m, load, cell_of, pts, np.zeros(npts),
                       gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    _, st2 = p2.forward(np.log(a2))
    prob = MisfitProblem(gpu, cells, m, load, cell_of, pts, st2["u"],
                         gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64, rtol=rtol)
    return prob, np.log(a)


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_gradient_matches_central_differences(gpu, precision):
    prob, theta = _problem(gpu, precision, rtol=1e-14)
    J, state = prob.forward(theta)
    grad = prob.gradient(theta, state)
    rng = np.random.default_rng(5)
    h = 1e-6
    for t in range(4):
        d = rng.standard_normal(theta.shape)
        fd = (prob.forward(theta + h * d)[0] - prob.forward(theta - h * d)[0]) / (2 * h)
        ad = float(grad @ d)
        scale = float(np.abs(grad * d).sum())
        assert abs(fd - ad) <= 1e-6 * scale, (t, fd, ad, scale)
        if abs(fd) >= 0.1 * scale:
            assert abs(fd - ad) <= 1e-6 * abs(fd), (t, fd, ad)


def test_gradient_at_adjoint_benchmark_scale(gpu):
    """The adjoint benchmark's size: coarse 8^3 x depth 4 (2.1 M fine cells),
    log a ~ N(0,1) i.i.d. per fine cell (seed 4), 512 seeded observation
    points, data from a second seeded coefficient; central differences
    (h = 1e-6) along 16 seeded random directions against grad . d, with the
    stated tolerance 1e-6 of sum |g_i d_i| (over 2 M parameters a random
    direction cancels the directional derivative by ~1/sqrt(N), so it is the
    only scale that measures the gradient's error)."""
    prob, theta = _problem(gpu, "mixed", m=8, depth=4, npts=512, seed=4, rtol=1e-14)
    J, state = prob.forward(theta)
    grad = prob.gradient(theta, state)
    rng = np.random.default_rng(16)
    h = 1e-6
    worst = 0.0
    for t in range(16):
        d = rng.standard_normal(theta.shape)
        fd = (prob.forward(theta + h * d)[0] - prob.forward(theta - h * d)[0]) / (2 * h)
        ad = float(grad @ d)
        scale = float(np.abs(grad * d).sum())
        worst = max(worst, abs(fd - ad) / scale)
        assert abs(fd - ad) <= 1e-6 * scale, (t, fd, ad, scale)
    print(f"config-4 scale: 16 directions, max |fd - g.d| / sum|g d| = {worst:.2e}")


def test_mixed_gradient_matches_fp64_gradient(gpu):
    pm, theta = _problem(gpu, "mixed")
    pf, _ = _problem(gpu, "fp64")
    gm = pm.gradient(theta)
    gf = pf.gradient(theta)
    assert np.abs(gm - gf).max() <= 1e-8 * np.abs(gf).max()


def test_autograd_wrapper(gpu):
    import torch
    prob, theta = _problem(gpu, "mixed", m=2, depth=2, npts=16)
    fn = make_autograd(prob)
    th = torch.tensor(theta, requires_grad=True)
    J = fn(th)
    J.backward()
    grad = prob.gradient(theta)
    assert np.allclose(th.grad.numpy(), grad, rtol=1e-12, atol=0)


def test_gpu_gradient_matches_oracle_gradient(gpu, oracle_lib):
    from oracle import q1_adjoint
    prob, theta = _problem(gpu, "mixed", m=2, depth=2, npts=24)
    g_gpu = prob.gradient(theta)
    J_o, g_or = q1_adjoint.misfit(prob.cells, prob.m, theta, prob.load, prob.cell_of, prob.points, prob.data)
    J_g, _ = prob.forward(theta)
    assert abs(J_g - J_o) <= 1e-9 * abs(J_o)
    assert np.abs(g_gpu - g_or).max() <= 1e-8 * np.abs(g_or).max()
