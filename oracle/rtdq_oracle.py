"""FP64 CPU oracle, Raviart-Thomas x DQ0 pairing (numpy + scipy).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA path in tests/; the
product library never imports it.

Restates the reference's mixed local basis problem of the RT_DQ pairing
(konsim83/MPI-MSFEC, source/RT_DQ/rt_dq_basis.cc):
  fe = FE_RaviartThomas<3>(0) (sigma) x FE_DGQ<3>(0) (u)       :18-20
  setup_basis_dofs_div (:267-389): basis n has sigma . n on the boundary =
      the coarse RT function n (BasisRaviartThomas)
  assemble_system (:391-580): local matrix (A^-1 sigma, tau) - (div tau, u)
      + (v, div sigma) + (R u, v), R = ReactionRate = 0 (eqn_coeff_R.cc:7-14);
      is_laplace (rt_dq_parameters.h:38): basis n's right-hand side on the u
      rows is -+ 1/|K| (v, 1) (minus for the low faces n = 0, 2, 4)
  solve_iterative (:615-820): Schur complement CG whose right-hand side has its
      mean removed (:683-698): the local problem is a pure-Neumann one, the
      pressure is fixed up to a constant; restated here by a bordered direct
      solve with mean-zero pressure (sigma is unique either way)
  run (:1114-1216) then calls set_u_to_std (:1039-1044): the u block of every
      stored basis is overwritten by the constant 1 before the Galerkin product
  assemble_global_element_matrix (:822-914): 7 x 7 (length_system_basis =
      faces + 1, :38) with the test/trial vector of index i taken from basis
      i % 6 (:845, :855): sigma of basis i for i < 6, the u block of basis 0
      (= 1) for i = 6, against the unconstrained matrix; F_H[6] = 1 . (v, f)
Hence K_H[i][j] = sigma_i^T M sigma_j (i, j < 6), K_H[6][j] = -K_H[j][6] =
sum over fine cells of (B sigma_j)_c = the net outflow of sigma_j, K_H[6][6] =
0 (R = 0), F_H[6] = the integral of f over the coarse cell.
Fine DoFs per cell: faces in the Ned_RT numbering (x-, y-, z-faces), then
cells (lexicographic). Face DoF = flux in the positive axis direction.

Parity partially pinned: no reference test or fixture covers this pairing.
Pinned by known answers: constant diagonal coefficients give the coarse RT
functions, the multiscale solution converges to a closed-form solution in the
coarse mesh size, and the reference's own Schur-complement CG (restated in
tests/test_oracle_rtdq.py) gives this oracle's sigma.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import nedrt_oracle as NR

LOAD_ZERO, LOAD_CONSTANT, LOAD_SIN_PRODUCT = 0, 1, 2


def counts(n):
    _, NF = NR.counts(n)
    return NF, n ** 3


def cell_faces(n):
    _, fidx = NR.cell_dofs(n)
    return fidx


def element_matrices(h, ainv):
    """Per-cell RT0 mass with A^-1 [c,6,6] and the divergence row (+-1) of the 6 faces."""
    _, wts, E, CE, F, DF = NR.local_functions(h)
    Mf = np.einsum("q,iqa,cab,jqb->cij", wts, F, ainv, F)
    Bf = np.einsum("q,iq->i", wts, DF)  # integral of div psi_f over the cell: -1 low, +1 high
    return Mf, Bf


def assemble(n, size, ainv):
    """Unconstrained [[M, -B^T], [B, 0]] (scipy CSR), faces then cells."""
    h = np.asarray(size, dtype=np.float64) / n
    Mf, Bf = element_matrices(h, ainv)
    fidx = cell_faces(n)
    NF, NC = counts(n)
    c = np.arange(n ** 3)
    rows, cols, vals = [], [], []
    for a in range(6):
        for b in range(6):
            rows.append(fidx[:, a]); cols.append(fidx[:, b]); vals.append(Mf[:, a, b])
        rows.append(fidx[:, a]); cols.append(NF + c); vals.append(np.full(n ** 3, -Bf[a]))
        rows.append(NF + c); cols.append(fidx[:, a]); vals.append(np.full(n ** 3, Bf[a]))
    return sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(NF + NC, NF + NC)).tocsr()


def boundary_mask(n):
    NE, NF = NR.counts(n)
    return np.concatenate([NR.boundary_mask(n)[NE:], np.zeros(n ** 3, dtype=bool)])


def cell_load(n, origin, size, kind, params):
    """(v_c, f) for every fine cell (2x2x2 Gauss) of a scalar load: CONSTANT p0,
    SIN_PRODUCT p0 sin(p1 pi x) sin(p1 pi y) sin(p1 pi z)."""
    if kind == LOAD_ZERO:
        return np.zeros(n ** 3)
    h = np.asarray(size, dtype=np.float64) / n
    pts, wts, *_ = NR.local_functions(h)
    c = np.arange(n ** 3)
    ci = np.stack([c % n, (c // n) % n, c // (n * n)], 1).astype(np.float64)
    P = np.asarray(origin)[None, None, :] + (ci[:, None, :] + pts[None, :, :]) * h[None, None, :]
    if kind == LOAD_CONSTANT:
        f = np.full(P.shape[:2], params[0])
    else:
        w = params[1] * np.pi
        f = params[0] * np.sin(w * P[..., 0]) * np.sin(w * P[..., 1]) * np.sin(w * P[..., 2])
    return np.einsum("q,cq->c", wts, f)


def build_cell(origin, size, depth, ainv, load_kind=LOAD_ZERO, load_params=(0, 0, 0, 0)):
    """One coarse cell. Returns (Phi [6, NF+NC] as the reference stores it:
    sigma solved, u = 1; P [6, NC] the mean-zero local pressures; KH [7,7]; FH [7])."""
    n = 1 << int(depth)
    NF, NC = counts(n)
    A = assemble(n, size, ainv)
    bnd = boundary_mask(n)
    I = np.where(~bnd)[0]
    B = np.where(bnd)[0]
    h = np.asarray(size, dtype=np.float64) / n
    G = np.zeros((6, NF + NC))
    rhs = np.zeros((NF + NC, 6))
    vol_ratio = np.prod(h) / np.prod(np.asarray(size, dtype=np.float64))
    for f in range(6):
        G[f, :NF] = NR.coarse_face_dofs(n, f)
        rhs[NF:, f] = (1.0 if f & 1 else -1.0) * vol_ratio
    G[:, I] = 0.0
    R = rhs[I, :] - A[I][:, B] @ G[:, B].T
    # bordered system: the constant pressure spans the kernel of A_II
    AII = A[I][:, I].tocsc()
    nI = len(I)
    cel = np.where(I >= NF)[0]
    R[cel] -= R[cel].mean(0, keepdims=True)
    border = sp.coo_matrix((np.ones(len(cel)), (cel, np.zeros(len(cel), dtype=int))), shape=(nI, 1))
    K = sp.bmat([[AII, border], [border.T, None]]).tocsc()
    X = NR.solve_refined(K, np.vstack([R, np.zeros((1, 6))]))[:nI]
    Phi = G
    Phi[:, I] = X.T
    P = Phi[:, NF:].copy()
    Phi[:, NF:] = 1.0
    T = np.zeros((7, NF + NC))
    T[:6, :NF] = Phi[:, :NF]
    T[6, NF:] = 1.0
    KH = T @ (A @ T.T)
    FH = np.zeros(7)
    FH[6] = cell_load(n, origin, size, load_kind, load_params).sum()
    return Phi, P, KH, FH


def build(cells, ainv, load_kind=LOAD_ZERO, load_params=(0, 0, 0, 0), want_phi=True):
    """Batch over coarse cells; ainv [sum n^3, 3, 3]."""
    KH, FH, PH = [], [], []
    off = 0
    for c in cells:
        n = 1 << int(c["depth"])
        sl = slice(off, off + n ** 3)
        off += n ** 3
        phi, _, kh, fh = build_cell(c["origin"], c["size"], c["depth"], ainv[sl], load_kind, load_params)
        KH.append(kh)
        FH.append(fh)
        if want_phi:
            PH.append(phi)
    return {"KH": np.array(KH), "FH": np.array(FH), "Phi": PH if want_phi else None}
