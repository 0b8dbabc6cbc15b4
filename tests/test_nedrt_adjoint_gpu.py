"""Ned_RT adjoint (msfec_nedrt_backward) against the FP64 oracle gradient, central
finite differences of the GPU forward path, and the FP64 GPU path.

Problem: coarse 2^3 x depth 2 on the unit cube, tensor A^-1 and B of the
Ned_RT workload scaled by exp(-ta), exp(tb) per fine cell, vector trig load,
J = 1/2 sum_k |u_h(x_k) - d_k|^2 at 40 points. The coarse problem (assembly,
solve, transposed adjoint solve) is the harness's (scipy). Stated tolerances:
  GPU vs oracle   |g - g_ref| <= 1e-8 max|g_ref|  (both gradients; on the 2^3
                  grid the A gradient vanishes for this divergence-free load,
                  so it is compared against the B gradient's scale; the last
                  test runs coarse 3^3, where it does not vanish)
  FD (h = 1e-5)   |fd - g.d| <= 1e-6 sum|g_i d_i| (cancellation-aware)
  mixed vs FP64   1e-8 relative
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import workloads

pytestmark = pytest.mark.gpu


class NedRTMisfit:
    def __init__(self, gpu, m=2, depth=2, seed=5, npts=40, precision="mixed"):
        from oracle import nedrt_adjoint as NA
        from oracle import nedrt_oracle as N
        self.gpu, self.N, self.NA = gpu, N, NA
        self.m, self.depth = m, depth
        self.cells, self.ainv6, self.bdiv, self.load = workloads.nedrt_tensor(m=m, depth=depth, seed=seed)
        rng = np.random.default_rng(1)
        self.pts = rng.uniform(0.02, 0.98, (npts, 3))
        ci = np.minimum((self.pts * m).astype(int), m - 1)
        self.cell_of = (ci[:, 0] + m * (ci[:, 1] + m * ci[:, 2])).astype(np.int32)
        self.data = rng.standard_normal((npts, 3)) * 0.1
        self.h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
        self.g, self.cb = NA.coarse_maps(m)
        self.I = np.where(~self.cb)[0]

    def coefs(self, ta, tb):
        return self.ainv6 * np.exp(-ta)[:, None], self.bdiv * np.exp(tb)

    def forward(self, ta, tb):
        N, m = self.N, self.m
        a6, b = self.coefs(ta, tb)
        KH, FH, rep, st = self.h.nedrt_build(self.cells, a6, b, self.load)
        assert st == self.gpu.SUCCESS and rep["converged"].all()
        n = 1 << self.depth
        NE, NF = N.counts(n)
        nc = self.cb.size
        K = sp.coo_matrix((KH.ravel(), (np.repeat(self.g, 18, axis=1).ravel(), np.tile(self.g, (1, 18)).ravel())),
                          shape=(nc, nc)).tocsr()
        F = np.zeros(nc)
        np.add.at(F, self.g.ravel(), FH.ravel())
        lu = spla.splu(K[self.I][:, self.I].tocsc())
        U = np.zeros(nc)
        U[self.I] = lu.solve(F[self.I])
        Phi = list(self.h.nedrt_basis().reshape(m ** 3, 18, NE + NF))
        u, jac = self.NA.eval_u(self.cells, Phi, U, self.g, m, self.cell_of, self.pts, with_jac=True)
        r = u - self.data
        return 0.5 * float(np.sum(r ** 2)), (U, r, jac, Phi, lu, NE, NF)

    def gradient(self, ta, tb):
        J, state = self.forward(ta, tb)
        ga, gb = self.backward(ta, tb, state)
        return J, ga, gb

    def backward(self, ta, tb, state):
        """dJ/dta, dJ/dtb through msfec_nedrt_backward, reusing the basis of the
        forward build (the last Ned_RT build on this handle)."""
        m = self.m
        U, r, jac, Phi, lu, NE, NF = state
        e_cell = np.zeros((m ** 3, NF))
        for p in range(len(self.pts)):
            for fi, d, w in jac[p]:
                e_cell[self.cell_of[p], fi] += r[p, d] * w
        dJdU = np.zeros(self.cb.size)
        for c in range(m ** 3):
            for j in range(6):
                dJdU[self.g[c, 12 + j]] += e_cell[c] @ Phi[c][12 + j, NE:]
        lam = np.zeros(self.cb.size)
        lam[self.I] = lu.solve(dJdU[self.I], trans="T")
        a6, b = self.coefs(ta, tb)
        ga, gb = self.h.nedrt_backward(self.cells, a6, b, self.load, U[self.g], lam[self.g], self.cell_of, self.pts,
                                       r, reuse_basis=True)
        return ga, gb

    def oracle(self, ta, tb):
        ainv = self.N.sym6_to_ainv(self.ainv6)
        return self.NA.misfit(self.cells, self.m, ainv, self.bdiv, ta, tb, self.load.kind, list(self.load.params),
                              self.cell_of, self.pts, self.data)


def make_nedrt_autograd(P):
    """torch.autograd.Function (ta, tb) -> J over the C ABI forward/backward
    pair (test harness only): forward = msfec_nedrt_build + coarse solve +
    misfit, backward = msfec_nedrt_backward on the forward's basis."""
    import torch

    class NedRTMisfitFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, ta, tb):
            ta_np, tb_np = ta.detach().cpu().double().numpy(), tb.detach().cpu().double().numpy()
            J, state = P.forward(ta_np, tb_np)
            ctx.args = (ta_np, tb_np, state)
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            ga, gb = P.backward(*ctx.args)
            return torch.from_numpy(ga) * gout, torch.from_numpy(gb) * gout

    return NedRTMisfitFn.apply


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_nedrt_gradient_matches_oracle(gpu, precision):
    P = NedRTMisfit(gpu, precision=precision)
    rng = np.random.default_rng(7)
    ta = 0.3 * rng.standard_normal(P.bdiv.size)
    tb = 0.3 * rng.standard_normal(P.bdiv.size)
    J, ga, gb = P.gradient(ta, tb)
    Jr, gar, gbr = P.oracle(ta, tb)
    assert abs(J - Jr) <= 1e-9 * abs(Jr)
    scale = np.abs(gbr).max()
    assert np.abs(gb - gbr).max() <= 1e-8 * scale, np.abs(gb - gbr).max() / scale
    assert np.abs(ga - gar).max() <= 1e-8 * scale
    print(f"{precision}: |gb - gb_ref| / max|gb_ref| = {np.abs(gb - gbr).max() / scale:.2e}, "
          f"max|ga| = {np.abs(ga).max():.1e}")


def test_nedrt_gradient_finite_differences_and_fp64(gpu):
    P = NedRTMisfit(gpu, precision="mixed")
    P64 = NedRTMisfit(gpu, precision="fp64")
    rng = np.random.default_rng(8)
    ta = 0.2 * rng.standard_normal(P.bdiv.size)
    tb = 0.2 * rng.standard_normal(P.bdiv.size)
    J, ga, gb = P.gradient(ta, tb)
    _, ga64, gb64 = P64.gradient(ta, tb)
    assert np.abs(gb - gb64).max() <= 1e-8 * np.abs(gb64).max()
    hs = 1e-5
    for trial in range(3):
        d = rng.standard_normal(tb.size)
        Jp = P64.forward(ta, tb + hs * d)[0]
        Jm = P64.forward(ta, tb - hs * d)[0]
        fd = (Jp - Jm) / (2 * hs)
        assert abs(fd - gb @ d) <= 1e-6 * np.abs(gb * d).sum(), (trial, fd, gb @ d)
        d = rng.standard_normal(ta.size)
        fda = (P64.forward(ta + hs * d, tb)[0] - P64.forward(ta - hs * d, tb)[0]) / (2 * hs)
        assert abs(fda - ga @ d) <= 1e-6 * np.abs(gb * d).sum()


def test_nedrt_gradient_nonvanishing_A_matches_oracle(gpu):
    """Coarse 3^3 x depth 2: the coarse solution has an edge part, so dJ/d log A
    does not vanish (max|g_A| ~ 3.5 % of max|g_B|); both gradients against the
    oracle, each to 1e-8 of its own scale."""
    P = NedRTMisfit(gpu, m=3, depth=2, seed=5, precision="mixed")
    rng = np.random.default_rng(9)
    ta = 0.3 * rng.standard_normal(P.bdiv.size)
    tb = 0.3 * rng.standard_normal(P.bdiv.size)
    J, ga, gb = P.gradient(ta, tb)
    Jr, gar, gbr = P.oracle(ta, tb)
    assert abs(J - Jr) <= 1e-9 * abs(Jr)
    assert np.abs(gar).max() > 1e-2 * np.abs(gbr).max()
    assert np.abs(ga - gar).max() <= 1e-8 * np.abs(gar).max(), np.abs(ga - gar).max() / np.abs(gar).max()
    assert np.abs(gb - gbr).max() <= 1e-8 * np.abs(gbr).max(), np.abs(gb - gbr).max() / np.abs(gbr).max()


def test_nedrt_autograd_wrapper(gpu):
    """The autograd wrapper returns the C ABI's J and gradients (two GPU runs:
    shared-memory atomics vary the last bits, hence 1e-9)."""
    import torch
    P = NedRTMisfit(gpu, precision="mixed")
    rng = np.random.default_rng(11)
    ta0 = 0.2 * rng.standard_normal(P.bdiv.size)
    tb0 = 0.2 * rng.standard_normal(P.bdiv.size)
    ta = torch.tensor(ta0, requires_grad=True)
    tb = torch.tensor(tb0, requires_grad=True)
    J = make_nedrt_autograd(P)(ta, tb)
    J.backward()
    J2, ga, gb = P.gradient(ta0, tb0)
    assert abs(float(J.detach()) - J2) <= 1e-9 * abs(J2)
    assert np.abs(tb.grad.numpy() - gb).max() <= 1e-9 * np.abs(gb).max()
    assert np.abs(ta.grad.numpy() - ga).max() <= 1e-9 * np.abs(gb).max()
