"""Test harness of the Q1 adjoint: misfit J of the coarse multiscale solution,
its gradient through msfec_q1_backward, and a torch.autograd.Function wrapper.

J(theta) = 1/2 sum_k (u_H(x_k) - d_k)^2, theta = log a per fine cell,
u_H = sum_i U_i phi_i, K_H U = F_H on a structured m^3 coarse grid of the unit
cube with homogeneous Dirichlet data (the reference's QMultiscale problem).
The coarse problem (assembly, solves, observation weights) lives here on the
host; the GPU builds the basis and the fine-scale gradient.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def coarse_system(m, KH):
    M1 = m + 1
    rows, cols, vals = [], [], []
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        nodes = [(i + (v & 1)) + M1 * ((j + ((v >> 1) & 1)) + M1 * (k + (v >> 2))) for v in range(8)]
        for u in range(8):
            for v in range(8):
                rows.append(nodes[u]); cols.append(nodes[v]); vals.append(KH[c, u, v])
    K = sp.coo_matrix((vals, (rows, cols)), shape=(M1 ** 3, M1 ** 3)).tocsr()
    idx = np.arange(M1 ** 3)
    i, j, k = idx % M1, (idx // M1) % M1, idx // (M1 * M1)
    interior = np.where((i > 0) & (j > 0) & (k > 0) & (i < m) & (j < m) & (k < m))[0]
    return K, interior


def cell_nodes(m):
    M1 = m + 1
    out = np.zeros((m ** 3, 8), dtype=np.int64)
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        out[c] = [(i + (v & 1)) + M1 * ((j + ((v >> 1) & 1)) + M1 * (k + (v >> 2))) for v in range(8)]
    return out


def global_rhs(m, FH):
    b = np.zeros((m + 1) ** 3)
    np.add.at(b, cell_nodes(m).ravel(), FH.ravel())
    return b


class MisfitProblem:
    """theta per fine cell: a = exp(theta) (scalar layout), or A_e = exp(theta_e)
    base_e for a tensor coefficient base (layout TENSOR: [fine, 6], GAUSS:
    [fine, 48])."""

    def __init__(self, msfec, cells, m, load, cell_of, points, data, precision, rtol=None, base=None, layout=0):
        self.msfec, self.cells, self.m, self.load = msfec, cells, m, load
        self.cell_of = np.asarray(cell_of, dtype=np.int32)
        self.points = np.asarray(points, dtype=np.float64)
        self.data = np.asarray(data, dtype=np.float64)
        self.base = None if base is None else np.asarray(base, dtype=np.float64)
        self.h = msfec.Handle(precision=precision, rtol=rtol, q1_coefficient=layout)
        self.nodes = cell_nodes(m)

    def forward(self, theta):
        """J and the state needed by the gradient."""
        a = np.exp(theta) if self.base is None else self.base * np.exp(theta)[:, None]
        KH, FH, rep, st = self.h.q1_build(self.cells, a, None, self.load)
        K, I = coarse_system(self.m, KH)
        Kii = spla.splu(K[I][:, I].tocsc())
        U = np.zeros((self.m + 1) ** 3)
        U[I] = Kii.solve(global_rhs(self.m, FH)[I])
        Ue = U[self.nodes]
        u = self.h.q1_eval_fine(Ue, self.cell_of, self.points)
        J = 0.5 * float(np.sum((u - self.data) ** 2))
        return J, {"a": a, "Ue": Ue, "u": u, "Kii": Kii, "I": I}

    def gradient(self, theta, state=None):
        if state is None:
            _, state = self.forward(theta)
        g = state["u"] - self.data
        nc = len(self.cells)
        # dJ/dU_i = sum_k g_k phi_i(x_k): unit weights per coarse vertex
        cvec = np.zeros((self.m + 1) ** 3)
        for v in range(8):
            w = np.zeros((nc, 8))
            w[:, v] = 1.0
            phik = self.h.q1_eval_fine(w, self.cell_of, self.points)
            np.add.at(cvec, self.nodes[self.cell_of, v], g * phik)
        lam = np.zeros_like(cvec)
        lam[state["I"]] = state["Kii"].solve(cvec[state["I"]])
        return self.h.q1_backward(self.cells, state["a"], None, self.load, state["Ue"], lam[self.nodes],
                                  self.cell_of, self.points, g, reuse_basis=True)


def make_autograd(problem):
    """torch.autograd.Function: theta (fine cells) -> J."""
    import torch

    class MisfitFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            th = theta.detach().cpu().double().numpy()
            J, state = problem.forward(th)
            ctx.save_for_backward(theta)
            ctx.state = state
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            (theta,) = ctx.saved_tensors
            grad = problem.gradient(theta.detach().cpu().double().numpy(), ctx.state)
            return torch.from_numpy(grad).to(theta.dtype) * gout

    return MisfitFn.apply
