"""CPU check of the faithful-iterative Ned_RT oracle mode
(oracle/nedrt_iterative.py: the reference's Schur-complement CG with ILU(0)
inner preconditioning and 1e-6 tolerances) against the direct oracle: the
reference's own default basis solve reaches the direct solution to its
tolerance. Stated bounds (measured values in brackets, coarse cell of depth 2):
primary block of every basis <= 2e-6 relative [<= 5.9e-7], whole basis vector
<= 5e-5 [<= 1.1e-5], K_H <= 1e-5 relative to max |K_H|."""
import numpy as np

import workloads
from oracle import nedrt_iterative as NI
from oracle import nedrt_oracle as N


def test_faithful_iterative_mode_reaches_the_direct_oracle():
    cells, ainv6, bdiv, _ = workloads.nedrt_tensor(m=1, depth=2, seed=3)
    c = cells[0]
    ainv = N.sym6_to_ainv(ainv6)
    Phi, KH, _ = N.build_cell(c["origin"], c["size"], 2, ainv, bdiv)
    Pf, its = NI.build_cell_faithful(c["origin"], c["size"], 2, ainv, bdiv)
    assert max(its) < 50
    NE, NF = N.counts(4)
    for b in range(18):
        blk = slice(0, NE) if b < 12 else slice(NE, NE + NF)
        assert np.abs(Pf[b, blk] - Phi[b, blk]).max() <= 2e-6 * np.abs(Phi[b, blk]).max(), b
        assert np.abs(Pf[b] - Phi[b]).max() <= 5e-5 * np.abs(Phi[b]).max(), b
    # block Galerkin of the faithful basis (primary blocks, unconstrained operator)
    A = N.assemble(4, c["size"], ainv, bdiv)
    P = np.zeros_like(Pf)
    P[:12, :NE] = Pf[:12, :NE]
    P[12:, NE:] = Pf[12:, NE:]
    KHf = P @ (A @ P.T)
    assert np.abs(KHf - KH).max() <= 1e-5 * np.abs(KH).max()


def test_ilu0_is_exact_on_a_tridiagonal_pattern():
    """ILU(0) of a matrix whose LU factors have no fill-in is its exact LU."""
    n = 12
    A = np.diag(np.full(n, 4.0)) + np.diag(np.full(n - 1, -1.0), 1) + np.diag(np.full(n - 1, -1.5), -1)
    L, U = NI.ilu0(A)
    assert np.abs((L @ U).toarray() - A).max() <= 1e-14
