"""Faithful-iterative mode of the Ned_RT and Q_Ned oracles (TEST
INFRASTRUCTURE ONLY: the checker of the CUDA path in tests/; the product
library never imports it).

Restates the reference's default local solver of both mixed pairings,
NedRTBasis::solve_iterative (konsim83/MPI-MSFEC,
source/Ned_RT/ned_rt_basis.cc:637-830) and QNedBasis::solve_iterative
(source/Q_Ned/q_ned_basis.cc:628-790, the same scheme), on the interior DoFs
of one coarse cell (the constrained boundary DoFs carry the coarse data, as
distribute_local_to_global and distribute leave them):
  - blocks of the interior system: M = block(0,0) (first field: Ned_RT sigma
    edges / Q_Ned sigma vertices), B01 = block(0,1), B10 = block(1,0),
    B11 = block(1,1) (the unconstrained assembly of the oracle restricted to
    interior rows and columns);
  - M^-1 (InverseMatrix, include/linear_algebra/inverse_matrix.tpp:21-40):
    GMRES to 1e-6 * |src| preconditioned by ILU(0) of M
    (LocalInnerPreconditioner<3> = SparseILU, preconditioner.h:62-67);
  - Schur operator S x = B10 M^-1 B01 x - B11 x
    (schur_complement.tpp:69-84), right-hand side B10 M^-1 f - g
    (ned_rt_basis.cc:716-721), CG to 1e-6 * |schur rhs| (:723-724);
  - its preconditioner (:756-779): at most 14 CG steps (1e-6 relative) on the
    approximate Schur complement B10 ILU(M)^-1 B01 - B11
    (approximate_schur_complement.tpp:32-41, approximate_inverse.tpp:23-40);
  - first field = M^-1 (f - B01 u) (:807-813).
The iterates follow the same algorithm and tolerances; they are not bit for
bit deal.II's (its GMRES and ILU implementations are not restated line by
line). The point of this mode: the reference's own basis functions are
accurate to about the 1e-6 tolerances above, and the direct oracle (and the
GPU path, at 1e-14 relative residual) is the limit they approach. Use it as
the interior_solver of nedrt_oracle.build_cell / qned_oracle.build_cell.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla



def ilu0(A):
    """ILU(0) of a CSR matrix on its own sparsity pattern (deal.II SparseILU
    with default additional data). Returns (L unit lower, U upper) as CSR."""
    A = sp.csr_matrix(A, dtype=np.float64)
    A.sort_indices()
    n = A.shape[0]
    rows = [dict(zip(A.indices[A.indptr[i]:A.indptr[i + 1]], A.data[A.indptr[i]:A.indptr[i + 1]])) for i in range(n)]
    for i in range(n):
        ri = rows[i]
        for k in sorted(c for c in ri if c < i):
            rk = rows[k]
            ri[k] /= rk[k]
            lik = ri[k]
            for j, v in rk.items():
                if j > k and j in ri:
                    ri[j] -= lik * v
    Lr, Lc, Lv, Ur, Uc, Uv = [], [], [], [], [], []
    for i, ri in enumerate(rows):
        for j, v in ri.items():
            if j < i:
                Lr.append(i); Lc.append(j); Lv.append(v)
            else:
                Ur.append(i); Uc.append(j); Uv.append(v)
        Lr.append(i); Lc.append(i); Lv.append(1.0)
    L = sp.csr_matrix((Lv, (Lr, Lc)), shape=(n, n))
    U = sp.csr_matrix((Uv, (Ur, Uc)), shape=(n, n))
    return L, U


def _ilu_apply(L, U):
    def apply(v):
        y = spla.spsolve_triangular(L, v, lower=True, unit_diagonal=True)
        return spla.spsolve_triangular(U, y, lower=False)
    return apply


def _cg(apply_A, b, apply_P, rtol, maxiter):
    """Preconditioned CG from x0 = 0, stopping at |r| <= rtol |b| (the
    unpreconditioned residual, as deal.II's SolverControl checks it) or after
    maxiter steps (the reference's approximate inverses catch NoConvergence
    and keep the last iterate)."""
    x = np.zeros_like(b)
    r = b.copy()
    tol = rtol * np.linalg.norm(b)
    if np.linalg.norm(r) <= tol:
        return x, 0
    z = apply_P(r)
    p = z.copy()
    rz = r @ z
    for it in range(1, maxiter + 1):
        Ap = apply_A(p)
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        if np.linalg.norm(r) <= tol:
            return x, it
        z = apply_P(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, maxiter


def faithful_solve(A_II, NEi, rhs):
    """Solve the interior block system A_II x = rhs (first field first: NEi
    DoFs) by the reference's Schur-complement scheme. Returns (x, Schur
    iterations)."""
    M = A_II[:NEi][:, :NEi].tocsr()
    B01 = A_II[:NEi][:, NEi:].tocsr()
    B10 = A_II[NEi:][:, :NEi].tocsr()
    B11 = A_II[NEi:][:, NEi:].tocsr()
    L, U = ilu0(M)
    ilu = _ilu_apply(L, U)
    ilu_op = spla.LinearOperator(M.shape, matvec=ilu)

    def Minv(v):
        if not np.any(v):
            return np.zeros_like(v)
        x, _ = spla.gmres(M, v, rtol=1e-6, atol=0.0, restart=30, maxiter=max(M.shape[0], 1000), M=ilu_op)
        return x

    def schur(x):
        return B10 @ Minv(B01 @ x) - B11 @ x

    def approx_schur(x):
        return B10 @ ilu(B01 @ x) - B11 @ x

    def precond(v):
        y, _ = _cg(approx_schur, v, lambda w: w, 1e-6, 14)
        return y

    f, g = rhs[:NEi], rhs[NEi:]
    schur_rhs = B10 @ Minv(f) - g
    # S is negative definite (-(C^T M^-1 C + D)); CG runs on it as the reference does
    u, its = _cg(schur, schur_rhs, precond, 1e-6, B10.shape[0] + B01.shape[1])
    sigma = Minv(f - B01 @ u)
    return np.concatenate([sigma, u]), its


def interior_solver(A_II, n_first, R):
    """Solve A_II X = R column by column with the reference's scheme (first
    field: the leading n_first interior DoFs). Returns X; the Schur iteration
    counts of the last call are kept in interior_solver.iterations."""
    cols, its = [], []
    for k in range(R.shape[1]):
        x, it = faithful_solve(A_II, n_first, np.asarray(R[:, k]).ravel())
        cols.append(x)
        its.append(it)
    interior_solver.iterations = its
    return np.array(cols).T
