"""FP64 CPU oracle of the Ned_RT adjoint gradient (TEST INFRASTRUCTURE ONLY).

Multiscale Nedelec x Raviart-Thomas solution on a structured m^3 coarse grid
of the unit cube with essential conditions (coarse tangential edges and normal
faces on the boundary are zero). Parameters: two log-scales per fine cell,
A_e = exp(ta_e) Ahat_e (A^-1 scaled by exp(-ta_e)) and B_e = exp(tb_e) Bhat_e.
Misfit of the coarse
multiscale u field (face bases' u-blocks weighted by the coarse solution, as
NedRTBasis::set_global_weights forms it, source/Ned_RT/ned_rt_basis.cc:
1155-1181) at points: J = 1/2 sum_k |u_h(x_k) - d_k|^2.

With K_H = P^T A P (primary blocks P of the basis, the reference's
assemble_global_element_matrix, ned_rt_basis.cc:849-948), F_H = P_u^T b,
s = P U, t = P lambda (lambda = K^-T dJ/dU), e = dJ/du_h (fine face vector),
dA/dta_e = -M_e (edge mass of cell e), dA/dtb_e = +D_e (div-div of cell e):

  dJ/dta_e = + t_s^T M_e s_s + sum_j eta_j,s^T M_e phi_j,s    (s: sigma block)
  dJ/dtb_e = - t_u^T D_e s_u - sum_j eta_j,u^T D_e phi_j,u    (u: u block)
  eta_j = A_II^-T (Pi_j w_j)_I,
  w_j = -lambda_j A s - U_j A^T t + [j face] (lambda_j b + U_j e),

Pi_j the primary block of basis j. eta_j is linear in (lambda_j, U_j) with
four distinct right-hand sides per cell (edge / face bases x lambda / U), so
four transposed local solves per cell (A^T = S A S, S = +1 on edges, -1 on
faces). The reference has no adjoint; this is the derivative of its Ned_RT
path restated here. For the divergence-free trig load on a coarse 2^3 grid the
coarse solution has no edge part and does not depend on A (dJ/dta vanishes; B
carries the sensitivity); on a 3^3 grid it has one and dJ/dta does not vanish.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import nedrt_oracle as N


def coarse_maps(m):
    """Global coarse DoF indices [m^3, 18] (12 lines in GeometryInfo order, then
    6 faces) and the boundary mask of the coarse DoFs (edges then faces)."""
    eidx, fidx = N.cell_dofs(m)
    NEc, _ = N.counts(m)
    # cell_dofs lists edges as x(j,k),(j+1,k),(j,k+1),(j+1,k+1), y(i,k)..., z(i,j)...
    local_of = {}
    for l, (d, (p, q)) in enumerate(N.COARSE_LINES):
        local_of[l] = 4 * d + p + 2 * q
    g = np.zeros((m ** 3, 18), dtype=np.int64)
    for l in range(12):
        g[:, l] = eidx[:, local_of[l]]
    for f, (d, a) in enumerate(N.COARSE_FACES):
        g[:, 12 + f] = NEc + fidx[:, 2 * d + a]
    return g, N.boundary_mask(m)


def _point_faces(cell, n, t):
    """Fine cell (lexicographic), its 6 face indices (within the face block)
    and the RT0 weights w[d][side] so that u_d(x) = sum_side w * u_face."""
    s = np.asarray(t) * n
    f = np.minimum(np.floor(s).astype(int), n - 1)
    tau = s - f
    c = f[0] + n * (f[1] + n * f[2])
    return c, tau


def eval_u(cells, Phi, U, g, m, cell_of, points, with_jac=False):
    """u_h at the points [np, 3]; optionally the per-point sparse derivative
    w.r.t. the fine face DoFs of its coarse cell: list of (face index, comp, w)."""
    out = np.zeros((len(points), 3))
    jac = []
    for p, x in enumerate(points):
        c = int(cell_of[p])
        n = 1 << int(cells["depth"][c])
        NE, NF = N.counts(n)
        h = np.asarray(cells["size"][c]) / n
        t = (np.asarray(x) - cells["origin"][c]) / cells["size"][c]
        fc, tau = _point_faces(c, n, t)
        _, fidx = N.cell_dofs(n)
        uf = sum(U[g[c, 12 + j]] * Phi[c][12 + j, NE:] for j in range(6))
        terms = []
        for d in range(3):
            o = [k for k in range(3) if k != d]
            area = h[o[0]] * h[o[1]]
            for side in range(2):
                w = (tau[d] if side else 1.0 - tau[d]) / area
                fi = fidx[fc, 2 * d + side]
                out[p, d] += w * uf[fi]
                terms.append((fi, d, w))
        jac.append(terms)
    return (out, jac) if with_jac else out


def misfit(cells, m, ainv_hat, bdiv_hat, ta, tb, load_kind, load_params, cell_of, points, data, gradient=True):
    """(J, dJ/dta, dJ/dtb) (gradients None without `gradient`) for a
    uniform-depth batch on the m^3 coarse grid."""
    depth = int(cells["depth"][0])
    n = 1 << depth
    NE, NF = N.counts(n)
    nf = n ** 3
    ainv = ainv_hat * np.exp(-ta)[:, None, None]
    bdiv = bdiv_hat * np.exp(tb)
    g, cb = coarse_maps(m)
    Ncoarse = cb.size
    Phi, KH, FH, Amat = [], [], [], []
    for c in range(m ** 3):
        sl = slice(c * nf, (c + 1) * nf)
        ph, kh, fh = N.build_cell(cells["origin"][c], cells["size"][c], depth, ainv[sl], bdiv[sl], load_kind,
                                  load_params)
        Phi.append(ph)
        KH.append(kh)
        FH.append(fh)
        Amat.append(N.assemble(n, cells["size"][c], ainv[sl], bdiv[sl]).tocsr())
    rows = np.repeat(g, 18, axis=1).ravel()
    cols = np.tile(g, (1, 18)).ravel()
    K = sp.coo_matrix((np.array(KH).ravel(), (rows, cols)), shape=(Ncoarse, Ncoarse)).tocsr()
    F = np.zeros(Ncoarse)
    np.add.at(F, g.ravel(), np.array(FH).ravel())
    I = np.where(~cb)[0]
    lu = spla.splu(K[I][:, I].tocsc())
    U = np.zeros(Ncoarse)
    U[I] = lu.solve(F[I])
    u, jac = eval_u(cells, Phi, U, g, m, cell_of, points, with_jac=True)
    r = u - data
    J = 0.5 * float(np.sum(r ** 2))
    if not gradient:
        return J, None, None
    # e = dJ/du_h per coarse cell (fine face vector), dJ/dU (face bases only)
    e_cell = [np.zeros(NF) for _ in range(m ** 3)]
    for p in range(len(points)):
        for fi, d, w in jac[p]:
            e_cell[int(cell_of[p])][fi] += r[p, d] * w
    dJdU = np.zeros(Ncoarse)
    for c in range(m ** 3):
        for j in range(6):
            dJdU[g[c, 12 + j]] += e_cell[c] @ Phi[c][12 + j, NE:]
    lam = np.zeros(Ncoarse)
    lam[I] = lu.solve(dJdU[I], trans="T")
    bnd = N.boundary_mask(n)
    Iin = np.where(~bnd)[0]
    S = np.r_[np.ones(NE), -np.ones(NF)]
    h = np.asarray(cells["size"][0]) / n
    eidx, _ = N.cell_dofs(n)
    ga = np.zeros_like(ta)
    gb = np.zeros_like(tb)
    _, fidx = N.cell_dofs(n)
    fsgn = np.array([-1.0, 1.0, -1.0, 1.0, -1.0, 1.0])
    for c in range(m ** 3):
        sl = slice(c * nf, (c + 1) * nf)
        A = Amat[c]
        Uc, Lc = U[g[c]], lam[g[c]]
        Ph = Phi[c]
        P = np.zeros_like(Ph)
        P[:12, :NE] = Ph[:12, :NE]
        P[12:, NE:] = Ph[12:, NE:]
        s, t = Uc @ P, Lc @ P
        b = np.zeros(NE + NF)
        b[NE:] = N.face_load(n, cells["origin"][c], cells["size"][c], load_kind, load_params)
        e = np.zeros(NE + NF)
        e[NE:] = e_cell[c]
        As, Att = A @ s, A.T @ t
        flu = spla.splu(A[Iin][:, Iin].tocsc())

        def eta(v, blk):
            w = np.zeros(NE + NF)
            if blk == "s":
                w[:NE] = v[:NE]
            else:
                w[NE:] = v[NE:]
            out = np.zeros(NE + NF)
            # A_II^T x = w_I  <=>  A_II (S x) = S w_I
            out[Iin] = S[Iin] * flu.solve(S[Iin] * w[Iin])
            return out

        eEl, eEU = eta(-As, "s"), eta(-Att, "s")
        eFl, eFU = eta(b - As, "u"), eta(e - Att, "u")
        PhEl, PhEU = Lc[:12] @ Ph[:12], Uc[:12] @ Ph[:12]
        PhFl, PhFU = Lc[12:] @ Ph[12:], Uc[12:] @ Ph[12:]
        Me, _, _ = N.element_matrices(h, ainv[sl], bdiv[sl])

        def q(x, y):
            return np.einsum("ea,eab,eb->e", x[eidx], Me, y[eidx])

        def qd(x, y):  # x_u^T D_e y_u = B_e / |K| div_e(x) div_e(y)
            dx = (x[NE:][fidx] * fsgn).sum(1)
            dy = (y[NE:][fidx] * fsgn).sum(1)
            return bdiv[sl] / np.prod(h) * dx * dy

        ga[sl] = q(t, s) + q(eEl, PhEl) + q(eEU, PhEU) + q(eFl, PhFl) + q(eFU, PhFU)
        gb[sl] = -(qd(t, s) + qd(eEl, PhEl) + qd(eEU, PhEU) + qd(eFl, PhFl) + qd(eFU, PhFU))
    return J, ga, gb
