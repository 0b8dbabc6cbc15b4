"""CPU checks of the cell-patch edge preconditioner of the Ned_RT solver
(nedrt_precond 0 on cells with a global MINRES workspace), restated in Python
from the kernel's index maps (csrc/nedrt_solver.cuh: nr_edge_line,
nr_edge_pos_in, nr_ainv_pq; csrc/nedrt_solve.cu: nr_cell_prep_kernel's patch
assembly) against explicit matrices built from the oracle:
  - the 12 x 12 block that the kernel assembles for a fine cell from the element
    edge masses of the fine cells around each of its edges equals the assembled
    edge mass M of the oracle restricted to that cell's edges;
  - the additive Schwarz operator over those blocks (Dirichlet rows and columns
    dropped), in the kernel's form X_c = L^-T L^-1 with L^-1 rounded to FP16,
    is symmetric positive definite on the interior edges, and
    preconditioned MINRES with it in the edge block needs fewer iterations than
    with diag(M)^-1 (same multilevel face block)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import workloads
from oracle import nedrt_oracle as N


def edge_line(l, ci, cj, ck):
    """nr_edge_line: edge l of fine cell (ci, cj, ck) as (direction, lattice point)."""
    p, a, b = l >> 2, l & 1, (l >> 1) & 1
    x = ci + (0 if p == 0 else a)
    y = cj + (0 if p == 1 else (a if p == 0 else b))
    z = ck + (0 if p == 2 else b)
    return p, x, y, z


def edge_pos_in(p, x, y, z, ci, cj, ck):
    """nr_edge_pos_in: position of the line among the cell's direction-p edges, or -1."""
    dx, dy, dz = x - ci, y - cj, z - ck
    if p == 0:
        ok, pos = dx == 0 and 0 <= dy <= 1 and 0 <= dz <= 1, dy + 2 * dz
    elif p == 1:
        ok, pos = dy == 0 and 0 <= dx <= 1 and 0 <= dz <= 1, dx + 2 * dz
    else:
        ok, pos = dz == 0 and 0 <= dx <= 1 and 0 <= dy <= 1, dx + 2 * dy
    return pos if ok else -1


def patch_block(n, Me, c, interior):
    """The kernel's assembly of fine cell c's 12 x 12 edge-mass block: for each
    interior edge l, the (up to) 4 fine cells around it, and in each of them the
    element entry between l and every interior edge m >= l the cell also has."""
    ci, cj, ck = c % n, (c // n) % n, c // (n * n)
    B = np.zeros((12, 12))
    for l in range(12):
        if not interior[l]:
            continue
        p, x, y, z = edge_line(l, ci, cj, ck)
        for s in range(4):
            a, b = s & 1, s >> 1
            qi = x if p == 0 else x - 1 + a
            qj = y if p == 1 else (y - 1 + a if p == 0 else y - 1 + b)
            qk = z if p == 2 else z - 1 + b
            if min(qi, qj, qk) < 0 or max(qi, qj, qk) >= n:
                continue
            q_cell = (qk * n + qj) * n + qi
            l4 = edge_pos_in(p, x, y, z, qi, qj, qk)
            for m in range(l, 12):
                if not interior[m]:
                    continue
                q, xm, ym, zm = edge_line(m, ci, cj, ck)
                m4 = edge_pos_in(q, xm, ym, zm, qi, qj, qk)
                if m4 < 0:
                    continue
                B[l, m] += Me[q_cell, 4 * p + l4, 4 * q + m4]
    return np.triu(B) + np.triu(B, 1).T


@pytest.fixture(scope="module")
def cell3():
    depth = 3
    cells, ainv6, bdiv, _ = workloads.nedrt_tensor(m=1, depth=depth, seed=7)
    n = 1 << depth
    h = cells["size"][0] / n
    ainv = N.sym6_to_ainv(ainv6)
    Me, _, _ = N.element_matrices(h, ainv, bdiv)
    A = N.assemble(n, cells["size"][0], ainv, bdiv).tocsr()
    NE, NF = N.counts(n)
    bnd = N.boundary_mask(n)
    eidx, fidx = N.cell_dofs(n)
    return depth, n, Me, A, NE, NF, bnd, eidx, fidx


def test_patch_block_equals_assembled_edge_mass(cell3):
    depth, n, Me, A, NE, NF, bnd, eidx, fidx = cell3
    M = A[:NE][:, :NE].toarray()
    for c in range(n ** 3):
        interior = ~bnd[eidx[c]]
        B = patch_block(n, Me, c, interior)
        ref = M[np.ix_(eidx[c], eidx[c])] * np.outer(interior, interior)
        assert np.abs(B - ref).max() <= 1e-12 * np.abs(ref).max(), c


def test_patch_schwarz_is_spd_and_cuts_minres_iterations(cell3):
    depth, n, Me, A, NE, NF, bnd, eidx, fidx = cell3
    I = np.where(~bnd)[0]
    Ie, If = I[I < NE], I[I >= NE]
    M, C, D = A[Ie][:, Ie], -A[Ie][:, If], A[If][:, If]
    ne = len(Ie)
    pos = -np.ones(NE, dtype=np.int64)
    pos[Ie] = np.arange(ne)
    # additive Schwarz operator over the fine-cell patches, as an explicit matrix
    rows, cols, vals = [], [], []
    for c in range(n ** 3):
        interior = ~bnd[eidx[c]]
        B = patch_block(n, Me, c, interior)
        k = np.where(interior)[0]
        # the kernel stores L^-1 (M_c = L L^T) in FP16 and applies X = L^-T L^-1
        Li = np.linalg.inv(np.linalg.cholesky(B[np.ix_(k, k)])).astype(np.float16).astype(np.float64)
        X = Li.T @ Li
        assert np.abs(X - np.linalg.inv(B[np.ix_(k, k)])).max() <= 1e-2 * np.abs(X).max()
        g = pos[eidx[c][k]]
        rows.append(np.repeat(g, len(k)))
        cols.append(np.tile(g, len(k)))
        vals.append(X.ravel())
    Pe = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(ne, ne)).tocsr()
    assert abs(Pe - Pe.T).max() <= 1e-12 * abs(Pe).max()
    assert spla.eigsh(Pe, k=1, which="SA", return_eigenvectors=False)[0] > 0
    # MINRES on the symmetric form with diag(S)^-1 on the faces (S = D + C^T diag(M)^-1 C)
    Asym = sp.bmat([[M, -C], [-C.T, -D]]).tocsr()
    S = D + C.T @ sp.diags(1.0 / M.diagonal()) @ C
    dS = 1.0 / S.diagonal()
    b = np.random.default_rng(1).standard_normal(Asym.shape[0])

    def iterations(edge):
        its = [0]
        P = spla.LinearOperator(Asym.shape, lambda v: np.concatenate([edge(v[:ne]), dS * v[ne:]]))
        spla.minres(Asym, b, M=P, rtol=1e-8, maxiter=5000, callback=lambda x: its.__setitem__(0, its[0] + 1))
        return its[0]

    diag_its = iterations(lambda v: v / M.diagonal())
    patch_its = iterations(lambda v: Pe @ v)
    assert patch_its < 0.8 * diag_its, (patch_its, diag_its)
