"""Standard fine-scale Ned_RT solve (msfec_nedrt_fine_solve: the reference's
NedRTStd, natural boundary conditions on every face) against the FP64
oracle's sparse direct solve of the same system, and the rotation symmetry of
the unit-cube problem at depth 4. Tolerance (stated): relative L2 difference
<= 1e-8 (stopping test: relative residual nedrt_rtol = 1e-14 of the symmetric
form; condition numbers up to ~1e5 at these sizes)."""
import numpy as np
import pytest

import workloads
from oracle import nedrt_oracle as NR
from test_oracle_nedrt import cyclic_image

pytestmark = pytest.mark.gpu


def _oracle(cells, ainv6, bdiv, load, depth):
    c = cells[0]
    return NR.standard_solve(c["origin"], c["size"], depth, NR.sym6_to_ainv(ainv6), bdiv, load.kind,
                             list(load.params))


@pytest.mark.parametrize("precision,depth", [("mixed", 3), ("fp64", 3), ("mixed", 2)])
def test_nedrt_fine_solve_matches_oracle(gpu, precision, depth):
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=depth, seed=7)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    x, rep, st = h.nedrt_fine_solve(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"] == 1
    xr = _oracle(cells, ainv6, bdiv, load, depth)
    n = 1 << depth
    bnd = NR.boundary_mask(n)
    assert np.abs(xr[bnd]).max() > 0  # natural conditions: boundary DoFs are unknowns
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)


def test_nedrt_fine_solve_depth4_symmetry_and_oracle(gpu):
    depth, n = 4, 16
    cells = workloads.coarse_grid(1, depth)
    ainv6 = np.tile([0.7, 0.7, 0.7, 0.0, 0.0, 0.0], (n ** 3, 1))
    bdiv = np.full(n ** 3, 1.3)
    load = gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    h = gpu.Handle()
    x, rep, st = h.nedrt_fine_solve(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS
    y = np.empty_like(x)
    y[cyclic_image(n)] = x
    assert np.linalg.norm(y - x) <= 1e-8 * np.linalg.norm(x)
    xr = _oracle(cells, ainv6, bdiv, load, depth)
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)


def test_nedrt_fine_solve_zero_load_and_invalid(gpu):
    cells, ainv6, bdiv, _ = workloads.nedrt_tensor(m=1, depth=2, seed=8)
    h = gpu.Handle()
    x, rep, st = h.nedrt_fine_solve(cells, ainv6, bdiv, gpu.make_load())
    assert st == gpu.SUCCESS and np.all(x == 0.0)
    bad = cells.copy()
    bad["depth"] = 5
    with pytest.raises(gpu.MsfecError):
        h.nedrt_fine_solve(bad, np.zeros((32 ** 3, 6)), np.ones(32 ** 3), gpu.make_load())
    neg = bdiv.copy()
    neg[3] = -1.0
    with pytest.raises(gpu.MsfecError):
        h.nedrt_fine_solve(cells, ainv6, neg, gpu.make_load())


def test_nedrt_fine_solve_analytic_solution(gpu):
    """Known answer (oracle's vec_trig_exact_dofs): A^-1 = 0.7 I, B = 1.3, the
    vector trig load with w = pi; at depth 4 the oracle's discretisation error
    is 6.9e-7 (edge DoFs) and 3.2e-3 (face DoFs) relative, and the GPU solve
    must show the same."""
    depth, n = 4, 16
    cells = workloads.coarse_grid(1, depth)
    ainv6 = np.tile([0.7, 0.7, 0.7, 0.0, 0.0, 0.0], (n ** 3, 1))
    load = gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    x, rep, st = gpu.Handle().nedrt_fine_solve(cells, ainv6, np.full(n ** 3, 1.3), load)
    assert st == gpu.SUCCESS
    xe = NR.vec_trig_exact_dofs(n, 1.0, 1.0, 1.0 / 0.7)
    NE, _ = NR.counts(n)
    es = np.linalg.norm(x[:NE] - xe[:NE]) / np.linalg.norm(xe[:NE])
    eu = np.linalg.norm(x[NE:] - xe[NE:]) / np.linalg.norm(xe[NE:])
    assert es < 2e-6 and eu < 5e-3, (es, eu)
