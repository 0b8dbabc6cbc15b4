"""CPU checks of the Q_Ned (Q1 x Nedelec) FP64 oracle and of the discrete
factorisations the CUDA path uses (restated here in Python):
  grad Q1 -> Nedelec edge DoFs = end - start (Grad incidence),
  curl Nedelec -> RT0 face fluxes = circulations (C incidence), hence
  Gm = M_N(I) Grad and Kc = C^T M_RT(A) C per fine cell."""
import numpy as np

from oracle import nedrt_oracle as NR
from oracle import qned_oracle as Q
import workloads


def grad_incidence():
    """12x8: edge (dir p, positions (a, b) on the other axes) = v(end) - v(start)."""
    G = np.zeros((12, 8))
    pairs = [(0, 0), (1, 0), (0, 1), (1, 1)]
    for p in range(3):
        o = [d for d in range(3) if d != p]
        for l, (a, b) in enumerate(pairs):
            for end, sg in ((0, -1.0), (1, 1.0)):
                c = [0, 0, 0]
                c[p], c[o[0]], c[o[1]] = end, a, b
                G[4 * p + l, c[0] + 2 * c[1] + 4 * c[2]] = sg
    return G


def curl_incidence():
    """6x12: flux of curl N_e through face (normal d, side s) = signed circulation."""
    C = np.zeros((6, 12))
    pairs = [(0, 0), (1, 0), (0, 1), (1, 1)]
    for d in range(3):
        o1, o2 = (d + 1) % 3, (d + 2) % 3  # e_o1 x e_o2 = e_d
        for s in range(2):
            f = 2 * d + s
            # counterclockwise seen from +e_d: +o1-edge at o2=0, +o2-edge at o1=1, -o1 at o2=1, -o2 at o1=0
            for p, fixed_other, sg in ((o1, 0, 1.0), (o2, 1, 1.0), (o1, 1, -1.0), (o2, 0, -1.0)):
                oth = [x for x in range(3) if x != p]
                pos = {d: s}
                q = o2 if p == o1 else o1
                pos[q] = fixed_other
                a, b = pos[oth[0]], pos[oth[1]]
                l = pairs.index((a, b))
                C[f, 4 * p + l] += sg
    return C


def test_discrete_factorisations_match_quadrature():
    rng = np.random.default_rng(3)
    h = np.array([0.3, 0.17, 0.55])
    pts, wts, V, GV, E, CE = Q.vertex_functions(h)
    _, _, _, _, F, _ = NR.local_functions(h)
    G = grad_incidence()
    # grad phi_v = sum_e G[e, v] N_e pointwise
    assert np.abs(np.einsum("ev,eqa->vqa", G, E) - GV).max() < 1e-12
    C = curl_incidence()
    # curl N_e = sum_f C[f, e] psi_f pointwise
    assert np.abs(np.einsum("fe,fqa->eqa", C, F) - CE).max() < 1e-12
    Qm, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    A = Qm @ np.diag(np.exp(rng.standard_normal(3))) @ Qm.T
    Mv, Gm, Kc = Q.element_matrices(h, np.array([0.7]), A[None])
    MN = np.einsum("q,iqa,jqa->ij", wts, E, E)
    MRT = np.einsum("q,iqa,ab,jqb->ij", wts, F, A, F)
    assert np.abs(Gm - MN @ G).max() < 1e-12 * np.abs(Gm).max()
    assert np.abs(Kc[0] - C.T @ MRT @ C).max() < 1e-12 * np.abs(Kc[0]).max()


def test_oracle_basis_properties():
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=2, seed=4)
    A = np.linalg.inv(NR.sym6_to_ainv(ainv6))
    binv = 1.0 / bdiv
    n = 4
    NV, NE = Q.counts(n)
    Phi, KH, FH = Q.build_cell(cells["origin"][0], cells["size"][0], 2, binv, A, load.kind, list(load.params))
    bnd = Q.boundary_mask(n)
    # boundary data reproduced
    for v in range(8):
        cv = Q.coarse_vertex_values(n, v)
        assert np.abs(Phi[v, :NV][bnd[:NV]] - cv[bnd[:NV]]).max() < 1e-14
    for l in range(12):
        ce = NR.coarse_edge_dofs(n, l)
        assert np.abs(Phi[8 + l, NV:][bnd[NV:]] - ce[bnd[NV:]]).max() < 1e-14
    # interior equations satisfied
    Am = Q.assemble(n, cells["size"][0], binv, A)
    I = np.where(~bnd)[0]
    assert np.all(np.isfinite(KH)) and np.abs(KH).max() > 0
    assert np.abs(FH[:8]).max() == 0.0 and np.abs(FH[8:]).max() > 0
    # partition of unity: sum of the vertex bases' sigma blocks is 1 (constant in the kernel of grad)
    assert np.abs(Phi[:8, :NV].sum(0) - 1.0).max() < 1e-10
    assert Am.shape == (NV + NE, NV + NE) and len(I) > 0


def test_committed_qned_fixture_reproduces():
    """The oracle against its committed K_H / F_H (tests/golden/make_golden.py)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "qned_tensor_m2_L2_seed4.npz"))
    cells, a6, binv, load = workloads.qned_tensor(m=2, depth=2, seed=4)
    res = Q.build(cells, binv, NR.sym6_to_ainv(a6), load.kind, list(load.params), want_phi=False)
    assert np.abs(res["KH"] - g["KH"]).max() <= 1e-9 * np.abs(g["KH"]).max()
    assert np.abs(res["FH"] - g["FH"]).max() <= 1e-9 * np.abs(g["FH"]).max()


def test_constant_diagonal_coefficients_give_the_standard_basis():
    """Known answer: with a constant diagonal A and constant B^-1 the vertex
    bases' sigma is the trilinear coarse function and the edge bases' u the
    coarse Nedelec function (any box); a full constant tensor breaks the
    latter (~5 %)."""
    n, size = 4, np.array([1.0, 0.8, 1.3])
    NV, _ = Q.counts(n)
    for A3, holds in ((np.diag([0.5, 1.0, 2.0]), True),
                      (np.array([[1.0, 0.3, 0.1], [0.3, 0.8, -0.2], [0.1, -0.2, 1.5]]), False)):
        Phi, _, _ = Q.build_cell(np.zeros(3), size, 2, np.full(n ** 3, 1.7), np.tile(A3, (n ** 3, 1, 1)))
        ev = max(np.abs(Phi[v, :NV] - Q.coarse_vertex_values(n, v)).max() for v in range(8))
        ee = max(np.abs(Phi[8 + l, NV:] - NR.coarse_edge_dofs(n, l)).max() / np.abs(NR.coarse_edge_dofs(n, l)).max()
                 for l in range(12))
        assert ev <= 1e-12
        assert (ee <= 1e-12) if holds else (ee > 1e-3), ee
