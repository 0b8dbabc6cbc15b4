"""CPU check of the faithful-iterative oracle mode (oracle/faithful_iterative.py:
the reference's Schur-complement CG with ILU(0) inner preconditioning and 1e-6
tolerances, the default local solver of its Ned_RT and Q_Ned bases) against
the direct oracles: the reference's own default basis solve reaches the
direct solution to its tolerance. Stated bounds (coarse cells of depth 2):
primary block of every basis <= 2e-6 relative, whole basis vector <= 5e-5,
K_H <= 1e-5 relative to max |K_H|."""
import numpy as np

import workloads
from oracle import faithful_iterative as FI
from oracle import nedrt_oracle as N
from oracle import qned_oracle as Q


def _check(Phi, Pf, KH, KHf, n_first_field, n_first_bases):
    for b in range(Phi.shape[0]):
        blk = slice(0, n_first_field) if b < n_first_bases else slice(n_first_field, Phi.shape[1])
        assert np.abs(Pf[b, blk] - Phi[b, blk]).max() <= 2e-6 * np.abs(Phi[b, blk]).max(), b
        assert np.abs(Pf[b] - Phi[b]).max() <= 5e-5 * np.abs(Phi[b]).max(), b
    assert np.abs(KHf - KH).max() <= 1e-5 * np.abs(KH).max()


def test_faithful_iterative_nedrt_reaches_the_direct_oracle():
    """Measured: primary blocks within 1.3e-7-5.9e-7, 6-7 Schur iterations."""
    cells, ainv6, bdiv, _ = workloads.nedrt_tensor(m=1, depth=2, seed=3)
    c = cells[0]
    ainv = N.sym6_to_ainv(ainv6)
    Phi, KH, _ = N.build_cell(c["origin"], c["size"], 2, ainv, bdiv)
    Pf, KHf, _ = N.build_cell(c["origin"], c["size"], 2, ainv, bdiv, interior_solver=FI.interior_solver)
    assert max(FI.interior_solver.iterations) < 50
    NE, _ = N.counts(4)
    _check(Phi, Pf, KH, KHf, NE, 12)


def test_faithful_iterative_qned_reaches_the_direct_oracle():
    cells, a6, binv, _ = workloads.qned_tensor(m=1, depth=2, seed=3)
    c = cells[0]
    a3 = N.sym6_to_ainv(a6)
    Phi, KH, _ = Q.build_cell(c["origin"], c["size"], 2, binv, a3)
    Pf, KHf, _ = Q.build_cell(c["origin"], c["size"], 2, binv, a3, interior_solver=FI.interior_solver)
    assert max(FI.interior_solver.iterations) < 50
    NV, _ = Q.counts(4)
    _check(Phi, Pf, KH, KHf, NV, 8)


def test_ilu0_is_exact_on_a_tridiagonal_pattern():
    """ILU(0) of a matrix whose LU factors have no fill-in is its exact LU."""
    n = 12
    A = np.diag(np.full(n, 4.0)) + np.diag(np.full(n - 1, -1.0), 1) + np.diag(np.full(n - 1, -1.5), -1)
    L, U = FI.ilu0(A)
    assert np.abs((L @ U).toarray() - A).max() <= 1e-14
