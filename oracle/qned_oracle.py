"""FP64 CPU oracle, Q1 x Nedelec pairing (numpy + scipy SuperLU).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA path in tests/; the
product library never imports it.

Restates the reference's mixed local basis problem of the Q_Ned pairing
(konsim83/MPI-MSFEC):
  fe = FE_Q<3>(1) (sigma) x FE_Nedelec<3>(0) (u)      source/Q_Ned/q_ned_basis.cc:18
  setup_basis_dofs_h1 (8 sets)    q_ned_basis.cc:223-290: sigma = coarse Q1
      function on the boundary, u x n = grad of it
  setup_basis_dofs_curl (12 sets) q_ned_basis.cc:293-354: sigma = 0, u x n =
      coarse Nedelec function
  assemble_system                  q_ned_basis.cc:360-560: local matrix
      (B^-1 sigma, tau) - (grad tau, u) + (grad sigma, v) + (A curl u, curl v)
      (+ (R u, v), R = 0); basis right-hand side (v, grad of the coarse Q1
      function) for the 8 H1 bases (full_rhs), 0 for the curl bases; global
      load (v, f)
  assemble_global_element_matrix  q_ned_basis.cc:841-940: primary blocks
      (sigma of H1 bases, u of curl bases) with the unconstrained matrix;
      F_H on the curl-basis rows
Coarse basis order: 8 vertices (GeometryInfo<3>: v = x + 2y + 4z), then 12
lines in GeometryInfo<3> line order.

Fine DoFs per cell (lexicographic): vertices (i + (n+1)(j + (n+1)k)), then
edges in the Ned_RT numbering (x-, y-, z-edges). Discrete facts used by the
GPU path and checked here: grad of a Q1 function lies in the lowest-order
Nedelec space with edge DoF = difference of the end values, and the curl of
a Nedelec function lies in RT0 with face flux = the circulation around the
face, so the element blocks factor as M_N(I) Grad and C^T M_RT(A) C.

Parity partially pinned: no reference test or fixture covers this pairing.
Pinned by known answers: constant diagonal coefficients give the trilinear /
coarse Nedelec functions, the multiscale solution converges to a closed-form
solution in the coarse mesh size, and the reference's own iterative solver
restated (faithful_iterative.py) reaches this oracle's basis to its 1e-6
tolerance.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import nedrt_oracle as NR

LOAD_VEC_ZERO, LOAD_VEC_TRIG = 0, 3


def counts(n):
    NE, _ = NR.counts(n)
    return (n + 1) ** 3, NE


def cell_dofs(n):
    """Vertex (8, GeometryInfo order) and edge (12) indices of every fine cell."""
    c = np.arange(n ** 3)
    i, j, k = c % n, (c // n) % n, c // (n * n)
    N1 = n + 1
    vidx = np.stack([(i + (v & 1)) + N1 * ((j + ((v >> 1) & 1)) + N1 * (k + (v >> 2))) for v in range(8)], 1)
    eidx, _ = NR.cell_dofs(n)
    return vidx, eidx


def vertex_functions(h):
    """Values and gradients of the 8 Q1 vertex functions at the 8 Gauss points."""
    pts, wts, E, CE, F, DF = NR.local_functions(h)
    V = np.zeros((8, 8))
    GV = np.zeros((8, 8, 3))
    for q, (x, y, z) in enumerate(pts):
        for v in range(8):
            a, b, c = v & 1, (v >> 1) & 1, v >> 2
            V[v, q] = NR._psi(a, x) * NR._psi(b, y) * NR._psi(c, z)
            GV[v, q] = [NR._dpsi(a) * NR._psi(b, y) * NR._psi(c, z) / h[0],
                        NR._psi(a, x) * NR._dpsi(b) * NR._psi(c, z) / h[1],
                        NR._psi(a, x) * NR._psi(b, y) * NR._dpsi(c) / h[2]]
    return pts, wts, V, GV, E, CE


def element_matrices(h, binv, a3):
    """Per-cell blocks: Mv [c,8,8] (B^-1 mass), Gm [12,8] ((N_e, grad phi_v)),
    Kc [c,12,12] ((A curl N, curl N))."""
    _, wts, V, GV, E, CE = vertex_functions(h)
    Mv = np.einsum("q,iq,jq->ij", wts, V, V)[None] * binv[:, None, None]
    Gm = np.einsum("q,eqa,vqa->ev", wts, E, GV)
    Kc = np.einsum("q,iqa,cab,jqb->cij", wts, CE, a3, CE)
    return Mv, Gm, Kc


def assemble(n, size, binv, a3):
    """Unconstrained block matrix [[Mv, -Gm^T], [Gm, Kc]] (scipy CSR)."""
    h = np.asarray(size, dtype=np.float64) / n
    Mv, Gm, Kc = element_matrices(h, binv, a3)
    vidx, eidx = cell_dofs(n)
    NV, NE = counts(n)
    nc = n ** 3
    rows, cols, vals = [], [], []
    for a in range(8):
        for b in range(8):
            rows.append(vidx[:, a]); cols.append(vidx[:, b]); vals.append(Mv[:, a, b])
        for e in range(12):
            rows.append(vidx[:, a]); cols.append(NV + eidx[:, e]); vals.append(np.full(nc, -Gm[e, a]))
            rows.append(NV + eidx[:, e]); cols.append(vidx[:, a]); vals.append(np.full(nc, Gm[e, a]))
    for e in range(12):
        for f in range(12):
            rows.append(NV + eidx[:, e]); cols.append(NV + eidx[:, f]); vals.append(Kc[:, e, f])
    return sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(NV + NE, NV + NE)).tocsr()


def boundary_mask(n):
    NV, NE = counts(n)
    N1 = n + 1
    idx = np.arange(NV)
    i, j, k = idx % N1, (idx // N1) % N1, idx // (N1 * N1)
    vb = (i == 0) | (j == 0) | (k == 0) | (i == n) | (j == n) | (k == n)
    eb = NR.boundary_mask(n)[:NE]
    return np.concatenate([vb, eb])


def coarse_vertex_values(n, v):
    """Coarse Q1 function v (BasisQ1, basis_q1.tpp) at the fine vertices."""
    N1 = n + 1
    idx = np.arange(N1 ** 3)
    t = np.stack([idx % N1, (idx // N1) % N1, idx // (N1 * N1)], 1) / n
    a, b, c = v & 1, (v >> 1) & 1, v >> 2
    return NR._psi(a, t[:, 0]) * NR._psi(b, t[:, 1]) * NR._psi(c, t[:, 2])


def grad_edge_dofs(n, vals):
    """Edge DoFs (line integrals along +axis) of grad of a vertex field: end - start."""
    N1 = n + 1
    out = []
    for d, i, j, k in NR.edge_geometry(n):
        s = i + N1 * (j + N1 * k)
        step = [1, N1, N1 * N1][d]
        out.append(vals[s + step] - vals[s])
    return np.concatenate(out)


def edge_load(n, origin, size, kind, params):
    """(N_e, f) for every fine edge (2x2x2 Gauss): the global load of the u block."""
    _, NE = counts(n)
    if kind == LOAD_VEC_ZERO:
        return np.zeros(NE)
    h = np.asarray(size, dtype=np.float64) / n
    pts, wts, E, CE, F, DF = NR.local_functions(h)
    _, eidx = cell_dofs(n)
    c = np.arange(n ** 3)
    ci = np.stack([c % n, (c // n) % n, c // (n * n)], 1).astype(np.float64)
    P = np.asarray(origin)[None, None, :] + (ci[:, None, :] + pts[None, :, :]) * h[None, None, :]
    w = params[1] * np.pi
    s = np.sin(w * P)
    f = params[0] * np.stack([s[..., 1] * s[..., 2], s[..., 2] * s[..., 0], s[..., 0] * s[..., 1]], -1)
    loc = np.einsum("q,eqa,cqa->ce", wts, E, f)
    out = np.zeros(NE)
    np.add.at(out, eidx.ravel(), loc.ravel())
    return out


def build_cell(origin, size, depth, binv, a3, load_kind=LOAD_VEC_ZERO, load_params=(0, 0, 0, 0),
               interior_solver=None):
    """One coarse cell. Returns (Phi [20, NV+NE], KH [20,20], FH [20]).
    interior_solver(A_II, n_interior_vertices, R) -> X replaces the direct
    solve of the interior system (faithful_iterative.interior_solver: the
    reference's iterative scheme, q_ned_basis.cc:628-790)."""
    n = 1 << int(depth)
    NV, NE = counts(n)
    A = assemble(n, size, binv, a3)
    bnd = boundary_mask(n)
    I = np.where(~bnd)[0]
    B = np.where(bnd)[0]
    G = np.zeros((20, NV + NE))
    rhs = np.zeros((NV + NE, 20))
    h = np.asarray(size, dtype=np.float64) / n
    _, Gm, _ = element_matrices(h, binv, a3)
    vidx, eidx = cell_dofs(n)
    for v in range(8):
        cv = coarse_vertex_values(n, v)
        G[v, :NV] = cv
        G[v, NV:] = grad_edge_dofs(n, cv)
        # (v, grad phi_v^coarse) on the edge rows: Gm applied to the vertex values
        loc = np.einsum("ev,cv->ce", Gm, cv[vidx])
        r = np.zeros(NE)
        np.add.at(r, eidx.ravel(), loc.ravel())
        rhs[NV:, v] = r
    for l in range(12):
        G[8 + l, NV:] = NR.coarse_edge_dofs(n, l)
    Phi = G.copy()
    Gb = G.copy()
    Gb[:, I] = 0.0
    R = rhs[I, :] - A[I][:, B] @ Gb[:, B].T
    if interior_solver is None:
        X = NR.solve_refined(A[I][:, I], R)
    else:
        X = interior_solver(A[I][:, I].tocsr(), int(np.sum(I < NV)), R)
    Phi = Gb
    Phi[:, I] = X.T
    P = np.zeros_like(Phi)
    P[:8, :NV] = Phi[:8, :NV]
    P[8:, NV:] = Phi[8:, NV:]
    KH = P @ (A @ P.T)
    bu = edge_load(n, origin, size, load_kind, load_params)
    FH = np.zeros(20)
    FH[8:] = Phi[8:, NV:] @ bu
    return Phi, KH, FH


def build(cells, binv, a3, load_kind=LOAD_VEC_ZERO, load_params=(0, 0, 0, 0), want_phi=True):
    """Batch over coarse cells; binv [sum n^3], a3 [sum n^3, 3, 3]."""
    KH, FH, PH = [], [], []
    off = 0
    for c in cells:
        n = 1 << int(c["depth"])
        sl = slice(off, off + n ** 3)
        off += n ** 3
        phi, kh, fh = build_cell(c["origin"], c["size"], c["depth"], binv[sl], a3[sl], load_kind, load_params)
        KH.append(kh)
        FH.append(fh)
        if want_phi:
            PH.append(phi)
    return {"KH": np.array(KH), "FH": np.array(FH), "Phi": PH if want_phi else None}
