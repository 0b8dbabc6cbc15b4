"""Stretched coarse cells (sides 1 : 0.45 : 1.7) for the three mixed-form
pairings against the FP64 oracle: the element operators take the fine-cell
sides from the cell record and the multilevel setup probes the Schur operator
through them. Tolerances as in the pairings' own parity tests (K_H, F_H
<= 1e-10 relative; Ned_RT with both face preconditioners)."""
import numpy as np
import pytest

import workloads
from oracle import nedrt_oracle as NR
from oracle import qned_oracle as Q
from oracle import rtdq_oracle as RQ

pytestmark = pytest.mark.gpu
TOL = 1e-10
SIZE = (1.0, 0.45, 1.7)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _stretch(cells):
    cells = cells.copy()
    cells["size"] = np.array(SIZE)
    return cells


@pytest.mark.parametrize("precond", (0, 1))
def test_nedrt_stretched(gpu, precond):
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=3, seed=31)
    cells = _stretch(cells)
    h = gpu.Handle(nedrt_precond=precond)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = NR.build(cells, NR.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params), want_phi=False)
    assert _rel(KH[0], ref["KH"][0]) <= TOL
    assert _rel(FH[0], ref["FH"][0]) <= TOL


def test_qned_stretched(gpu):
    cells, a6, binv, load = workloads.qned_tensor(m=1, depth=3, seed=32)
    cells = _stretch(cells)
    h = gpu.Handle()
    KH, FH, rep, st = h.qned_build(cells, a6, binv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = Q.build(cells, binv, NR.sym6_to_ainv(a6), load.kind, list(load.params), want_phi=False)
    assert _rel(KH[0], ref["KH"][0]) <= TOL
    assert _rel(FH[0], ref["FH"][0]) <= TOL


def test_rtdq_stretched(gpu):
    cells, ainv6, load = workloads.rtdq_tensor(m=1, depth=3, seed=33)
    cells = _stretch(cells)
    h = gpu.Handle()
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = RQ.build(cells, NR.sym6_to_ainv(ainv6), load.kind, list(load.params), want_phi=False)
    assert _rel(KH[0], ref["KH"][0]) <= TOL
    assert _rel(FH[0], ref["FH"][0]) <= TOL
