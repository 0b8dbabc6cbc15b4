"""CPU checks of the RT_DQ (Raviart-Thomas x DQ0) FP64 oracle and of the
discrete facts the CUDA path uses (restated here in Python): the RT0 mass in
factored form (same normal: A^-1_dd h_d^2 / (6|c|) (2,1); normals d != e:
A^-1_de h_d h_e / (4|c|)), the divergence row = net outflow of the 6 face
fluxes, compatibility of the pure-Neumann local problems, and the 7 x 7
Galerkin structure that follows from u = 1 in every stored basis."""
import numpy as np

import workloads
from oracle import nedrt_oracle as NR
from oracle import rtdq_oracle as RQ


def factored_mass(h, A):
    V = np.prod(h)
    M = np.zeros((6, 6))
    for d in range(3):
        for s in range(2):
            for e in range(3):
                for t in range(2):
                    if d == e:
                        M[2 * d + s, 2 * e + t] = A[d, d] * h[d] ** 2 / (6 * V) * (2.0 if s == t else 1.0)
                    else:
                        M[2 * d + s, 2 * e + t] = A[d, e] * h[d] * h[e] / (4 * V)
    return M


def test_factored_mass_and_divergence_match_quadrature():
    rng = np.random.default_rng(11)
    h = np.array([0.31, 0.12, 0.47])
    Qm, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    A = Qm @ np.diag(np.exp(rng.standard_normal(3))) @ Qm.T
    Mf, Bf = RQ.element_matrices(h, A[None])
    assert np.abs(Mf[0] - factored_mass(h, A)).max() < 1e-12 * np.abs(Mf[0]).max()
    assert np.allclose(Bf, [-1, 1, -1, 1, -1, 1], atol=1e-14)


def test_local_problems_compatible_and_solved():
    cells, ainv6, load = workloads.rtdq_tensor(m=1, depth=2, seed=5)
    ainv = NR.sym6_to_ainv(ainv6)
    n = 4
    NF, NC = RQ.counts(n)
    o, sz = cells["origin"][0], cells["size"][0]
    Phi, P, KH, FH = RQ.build_cell(o, sz, 2, ainv, load.kind, list(load.params))
    A = RQ.assemble(n, sz, ainv)
    bnd = RQ.boundary_mask(n)
    I = np.where(~bnd)[0]
    for b in range(6):
        # boundary fluxes of the coarse RT function b, total outflow -+1
        cf = NR.coarse_face_dofs(n, b)
        assert np.abs(Phi[b, :NF][bnd[:NF]] - cf[bnd[:NF]]).max() < 1e-15
        x = np.concatenate([Phi[b, :NF], P[b]])
        r = A @ x
        r[NF:] -= (1.0 if b & 1 else -1.0) / NC
        assert np.abs(r[I]).max() < 1e-12
        assert abs(P[b].mean()) < 1e-14  # mean-zero pressure (the reference's Schur correction)
        assert np.all(Phi[b, NF:] == 1.0)  # set_u_to_std
    # Galerkin structure: SPD sigma block, +-1 divergence coupling, zero (6, 6), F_H only on the u row
    assert np.abs(KH[:6, :6] - KH[:6, :6].T).max() < 1e-14 * np.abs(KH).max()
    assert np.linalg.eigvalsh(KH[:6, :6]).min() > 0
    assert np.allclose(KH[6, :6], [-1, 1, -1, 1, -1, 1], atol=1e-12)
    assert np.allclose(KH[:6, 6], -KH[6, :6], atol=1e-12)
    assert KH[6, 6] == 0.0
    assert np.all(FH[:6] == 0.0) and abs(FH[6]) > 0


def test_pressure_constant_does_not_change_sigma():
    """sigma of the singular local problem is unique: shifting the pressure
    by a constant leaves every interior equation satisfied."""
    cells, ainv6, _ = workloads.rtdq_tensor(m=1, depth=1, seed=6)
    ainv = NR.sym6_to_ainv(ainv6)
    n = 2
    NF, NC = RQ.counts(n)
    Phi, P, KH, FH = RQ.build_cell(cells["origin"][0], cells["size"][0], 1, ainv)
    A = RQ.assemble(n, cells["size"][0], ainv)
    I = np.where(~RQ.boundary_mask(n))[0]
    x0 = np.concatenate([Phi[3, :NF], P[3]])
    x1 = np.concatenate([Phi[3, :NF], P[3] + 7.5])
    assert np.abs((A @ x0 - A @ x1)[I]).max() < 1e-12


def test_reference_schur_cg_gives_the_oracle_sigma():
    """The reference's solve_iterative (rt_dq_basis.cc:615-820), restated: CG on
    the Schur complement S = B M^-1 B^T of the condensed system, right-hand side
    B M^-1 f - g with its mean removed (:683-698), zero start; then
    sigma = M^-1 (f + B^T u). Its sigma equals the oracle's (bordered, mean-zero
    pressure) to the CG tolerance, and its pressure is mean-zero as well."""
    import scipy.sparse.linalg as spla
    cells, ainv6, _ = workloads.rtdq_tensor(m=1, depth=2, seed=8)
    ainv = NR.sym6_to_ainv(ainv6)
    n = 4
    NF, NC = RQ.counts(n)
    Phi, P, _, _ = RQ.build_cell(cells["origin"][0], cells["size"][0], 2, ainv)
    A = RQ.assemble(n, cells["size"][0], ainv)
    bnd = RQ.boundary_mask(n)
    I = np.where(~bnd)[0]
    If, Ic = I[I < NF], I[I >= NF]
    M = A[If][:, If].tocsc()
    Bt = -A[If][:, Ic]          # face rows: -B^T
    B = A[Ic][:, If]
    Mlu = spla.splu(M)
    for b in range(6):
        G = np.zeros(NF + NC)
        G[:NF] = NR.coarse_face_dofs(n, b)
        G[I] = 0.0
        rhs = np.zeros(NF + NC)
        rhs[NF:] = (1.0 if b & 1 else -1.0) / NC
        r = rhs - A @ G
        f, g = r[If], r[Ic]
        s_rhs = B @ Mlu.solve(f) - g
        s_rhs -= s_rhs.mean()
        S = spla.LinearOperator((len(Ic), len(Ic)), matvec=lambda u: -(B @ Mlu.solve(Bt @ u)))
        u, info = spla.cg(S, s_rhs, rtol=1e-13, maxiter=2000)
        assert info == 0
        sigma = Mlu.solve(f + Bt @ u)
        assert np.abs(sigma - Phi[b, If]).max() <= 1e-10 * np.abs(Phi[b, :NF]).max()
        assert abs(u.mean()) <= 1e-10 * np.abs(u).max()
        assert np.abs(u - P[b][Ic - NF]).max() <= 1e-8 * np.abs(u).max()


def test_committed_rtdq_fixture_reproduces():
    """The oracle against its committed K_H / F_H (tests/golden/make_golden.py)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rtdq_tensor_m2_L2_seed6.npz"))
    cells, ainv6, load = workloads.rtdq_tensor(m=2, depth=2, seed=6)
    res = RQ.build(cells, NR.sym6_to_ainv(ainv6), load.kind, list(load.params), want_phi=False)
    assert np.abs(res["KH"] - g["KH"]).max() <= 1e-9 * np.abs(g["KH"]).max()
    assert np.abs(res["FH"] - g["FH"]).max() <= 1e-9 * np.abs(g["FH"]).max()


def test_constant_diagonal_coefficients_give_the_standard_basis():
    """Known answer: with a constant diagonal A^-1 the coarse RT0 function of
    face f has constant divergence and a curl-free A^-1 sigma, so it solves its
    local problem: sigma of every basis is the standard coarse RT function (any
    box); a full constant tensor breaks it (~12 %)."""
    n, size = 4, np.array([1.0, 0.8, 1.3])
    NF, _ = RQ.counts(n)
    for A3, holds in ((np.diag([0.5, 1.0, 2.0]), True),
                      (np.array([[1.0, 0.3, 0.1], [0.3, 0.8, -0.2], [0.1, -0.2, 1.5]]), False)):
        Phi, _, _, _ = RQ.build_cell(np.zeros(3), size, 2, np.tile(A3, (n ** 3, 1, 1)))
        e = max(np.abs(Phi[f, :NF] - NR.coarse_face_dofs(n, f)).max() / np.abs(NR.coarse_face_dofs(n, f)).max()
                for f in range(6))
        assert (e <= 1e-12) if holds else (e > 1e-3), e
